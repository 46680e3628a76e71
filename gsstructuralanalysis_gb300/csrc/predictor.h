// predictor.h -- learned arc-length predictor: last four path points projected on a reduced
// modal basis -> MLP -> correction of the cubic extrapolation of the path.
#pragma once

#include <vector>

#include "mlp.h"
#include "problem.h"

namespace klsa {

struct LearnedPredictor {
    Problem& P;
    MLP* net;                       // may be null: plain cubic extrapolation (ablation)
    int nm;
    DevBuf<double> Phi;             // n x nm, internal order, column j at j*n (orthonormal)
    std::vector<double> in_mu, in_sd, out_mu, out_sd;
    DevBuf<double> hist;            // 4 x n ring of converged points
    double histL[4] = {0, 0, 0, 0};
    std::vector<double> histq;      // 4 x nm projections
    int count = 0, head = 0;
    DevBuf<double> dq, part;        // device scratch for projections / GEMV coefficients
    DevBuf<float> feat;
    std::vector<double> hpart;

    LearnedPredictor(Problem& P, MLP* net, const double* modes_pub, int nm, const double* in_mu,
                     const double* in_sd, const double* out_mu, const double* out_sd);
    void reset() { count = 0; head = 0; }
    // record a converged point (device vector, internal order)
    void push(const double* dU, double L);
    // guess for the next point (needs 4 points); writes the device vector Ug (internal order)
    bool guess(double* dUg, double* Lg);

private:
    void project(const double* dU, double* q);
    int slot(int back) const { return (head - 1 - back + 8) & 3; }   // back = 0: newest
};

}  // namespace klsa
