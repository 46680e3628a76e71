// apalm.h -- the adaptive parallel arc-length method (gsAPALM) over the device arc-length solver.
//
// gsAPALM (gsALMSolvers/gsAPALM.hpp) computes a coarse path with the arc-length method
// ("initiation" jobs), then refines every interval of it by re-solving the interval with
// SubIntervals shorter steps ("correction" jobs), and queues the sub-intervals whose end does
// not meet the coarse solution within Tolerance, up to MaxLevel levels.  gsAPALMData
// (gsAPALMData.hpp) keeps per branch the two knot vectors of the path (curve time t and its
// parameter xi), the solutions and their levels, and the job queue.
//
// Here the jobs run on the device arc-length solver and every solution stays in HBM.  With one
// solver the schedule is the reference's single-process one (gsAPALM.hpp:430-472, 822-932): jobs
// run in queue order, so the points and their order are those of a one-process reference run.
// With W worker solvers (add_worker: each its own arc-length object on its own problem and
// stream) parallel_solve runs the reference's MPI schedule (gsAPALM.hpp:276-378): a job goes to
// every idle worker, each finished job is submitted and its worker refilled at once, with the
// jobs finishing in the order they were handed out; the workers run concurrently on the GPU,
// each driven by its own host thread.
#pragma once

#include <deque>
#include <map>
#include <memory>
#include <tuple>
#include <vector>

#include "problem.h"
#include "solvers.h"

namespace klsa {

struct APSolution {
    std::shared_ptr<DevBuf<double>> U;   // free dofs, internal order
    double L = 0.0;
};

// gsAPALMData (gsALMSolvers/gsAPALMData.hpp)
class APALMData {
public:
    using Job = std::tuple<int, double, APSolution, APSolution>;   // ID, length, start, previous

    int maxLevel = 5;           // option "MaxLevel"
    double tolerance = 1e-1;    // option "Tolerance"

    void addStartPoint(double time, const APSolution& s, bool priority = false);
    void appendPoint(bool priority = false);
    void appendData(double time, const APSolution& s, bool priority = false);
    void setData(const std::vector<double>& times, const std::vector<APSolution>& sols);
    void init();
    Job pop();
    bool referenceByID(int ID, APSolution& out);
    void submit(int ID, const std::vector<double>& distances, std::vector<APSolution> sols, double upper,
                double lower);
    void finishJob(int ID) { jobs_.erase(ID); }
    double jobStartTime(int ID) { return tmap_[std::get<0>(jobs_.at(ID))]; }
    std::pair<double, double> jobTimes(int ID);
    int jobLevel(int ID) { return std::get<2>(jobs_.at(ID)); }
    bool empty() const { return queue_.empty(); }
    void flat(std::vector<double>& t, std::vector<APSolution>& s, std::vector<int>& lv) const;
    void setLength(double dt) { dt_ = dt; }
    double getLength() const { return dt_; }

private:
    void buildMap();
    static void insertKnot(std::vector<double>& kv, double x);
    std::vector<double> t_, xi_;                       // knot vectors (sorted, with repeats)
    std::map<double, std::shared_ptr<APSolution>> sol_, prev_;
    std::map<double, int> lev_;
    std::map<double, double> tmap_, ximap_;
    std::deque<std::tuple<double, double, int>> queue_;
    std::map<int, std::tuple<double, double, int>> jobs_;
    int ID_ = 0;
    double dt_ = 1.0;
};

// one arc-length solver that runs jobs: its object, its problem (stream, device state) and scratch
struct APWorker {
    ALMGPU* alm;
    Problem* P;
    std::shared_ptr<DevBuf<double>> tmp;
};

// gsAPALM (gsALMSolvers/gsAPALM.hpp)
class APALM {
public:
    APALM(ALMGPU& alm, const Options& opt);
    // another solver for the interval corrections of parallel_solve (same method, options and
    // problem description as the first; MPI rank w + 1 of the reference's schedule)
    void add_worker(ALMGPU& alm, Problem& P);
    int workers() const { return (int)workers_.size(); }
    void initialize();                                          // gsAPALM.hpp:86-100
    void add_start(const double* d_U, double L, double dL);     // _initStart (:102-120)
    void serial_solve(int nsteps);                              // :122-220
    void parallel_solve();                                      // :430-472 (one worker), :276-378 (several)
    void solve(int nsteps);                                     // :822-932
    int branches() const { return (int)times_.size(); }
    int solutions(int b) const { return (int)times_.at(b).size(); }
    const APSolution& solution(int b, int k) const { return sols_.at(b).at(k); }
    double time(int b, int k) const { return times_.at(b).at(k); }
    int level(int b, int k) const { return levels_.at(b).at(k); }

private:
    APSolution copy_current() { return copy_current(workers_[0]); }
    APSolution copy_current(APWorker& w);                        // (solutionU, solutionL) of a worker's ALM
    APSolution copy_of(const double* d_U, double L) { return copy_of(workers_[0], d_U, L); }
    APSolution copy_of(APWorker& w, const double* d_U, double L);
    double distance_between(const APSolution& a, const APSolution& b) { return distance_between(workers_[0], a, b); }
    double distance_between(APWorker& w, const APSolution& a, const APSolution& b);   // distance(a - b)
    int step_retry_limit() const { return 60; }
    void initiation(const APALMData::Job& job, double startTime, double& distance, std::vector<APSolution>& sols,
                    bool& bifurcation);
    void correction(APWorker& w, const APALMData::Job& job, std::pair<double, double> interval,
                    const APSolution& reference, std::vector<double>& distances,
                    std::vector<APSolution>& stepSolutions, double& upper, double& lower);
    void parallel_solve_workers();
    void finalize();
    int first_nonempty_branch() const;
    bool data_empty() const;

    ALMGPU& alm_;
    Problem& P_;
    int maxIt_, subIntervals_, dataMaxLevel_;
    bool singularPoint_;
    double branchLengthMult_, bifLengthMult_, dataTol_;
    std::deque<std::tuple<APSolution, double, bool>> starts_;
    std::vector<APALMData> data_;
    std::vector<std::vector<APSolution>> sols_;
    std::vector<std::vector<double>> times_;
    std::vector<std::vector<int>> levels_;
    std::vector<APWorker> workers_;
};

}  // namespace klsa
