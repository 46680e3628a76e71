// predictor.h -- learned arc-length predictor: last four path points projected on a reduced
// modal basis -> MLP -> correction of the cubic extrapolation of the path.
#pragma once

#include <vector>

#include "mlp.h"
#include "problem.h"

namespace klsa {

struct LearnedPredictor {
    static constexpr int PCH = 16;  // chunks of the projection (partial sums per chunk and mode)

    Problem& P;
    MLP* net;                       // may be null: plain cubic extrapolation (ablation)
    int nm;
    DevBuf<double> Phi;             // n x nm, internal order, column j at j*n (orthonormal)
    DevBuf<double> stats;           // in_mu | in_sd | out_mu | out_sd (4 (nm + 1) + 2 (nm + 1))
    DevBuf<double> hist;            // 4 x n ring of converged points
    double histL[4] = {0, 0, 0, 0};
    DevBuf<double> qpart;           // 4 x PCH x nm ring of the points' projection partial sums
    DevBuf<double> corr;            // nm + 1: network correction (dq, dL), destandardised
    DevBuf<float> hid;              // hidden activations of the network (h1 + h2)
    double* corrL_host = nullptr;   // pinned copy of corr[nm]
    int count = 0, head = 0;

    LearnedPredictor(Problem& P, MLP* net, const double* modes_pub, int nm, const double* in_mu,
                     const double* in_sd, const double* out_mu, const double* out_sd);
    ~LearnedPredictor();
    LearnedPredictor(const LearnedPredictor&) = delete;
    LearnedPredictor& operator=(const LearnedPredictor&) = delete;
    void reset() { count = 0; head = 0; }
    // record a converged point (device vector, internal order); no host synchronisation
    void push(const double* dU, double L);
    // guess for the next point (needs 4 points); writes the device vector Ug (internal order).
    // With a network: one read of the load-factor correction (one stream synchronisation).
    bool guess(double* dUg, double* Lg);
    // the same guess without waiting for the network: Lg without the network's load correction,
    // which stays on the device at *Lcorr (null without a network)
    bool guess_deferred(double* dUg, double* Lg, const double** Lcorr);

private:
    bool launch_guess(double* dUg, double* Lcubic);
    int slot(int back) const { return (head - 1 - back + 8) & 3; }   // back = 0: newest
};

}  // namespace klsa
