// apalm.cpp -- gsAPALM / gsAPALMData over the device arc-length solver (see apalm.h).
#include "apalm.h"

#include <future>

#include <algorithm>
#include <cmath>
#include <numeric>
#include <stdexcept>

namespace klsa {

// ---- gsAPALMData (gsALMSolvers/gsAPALMData.hpp) ----------------------------------------------

// gsKnotVector::insert: sorted, repeats kept
void APALMData::insertKnot(std::vector<double>& kv, double x) {
    kv.insert(std::upper_bound(kv.begin(), kv.end(), x), x);
}

// gsAPALMData.hpp:77-95: one level-1 job per interval of the parameter knots
void APALMData::init() {
    queue_.clear();
    for (size_t k = 0; k + 1 < xi_.size(); ++k) queue_.push_back(std::make_tuple(xi_[k], xi_[k + 1], 1));
    buildMap();
}

// gsAPALMData.hpp:97-121
void APALMData::addStartPoint(double time, const APSolution& s, bool priority) {
    const double xi = 0.0;
    insertKnot(t_, time);
    insertKnot(xi_, xi);
    sol_.insert({xi, std::make_shared<APSolution>(s)});
    lev_.insert({xi, 0});
    prev_.insert({xi, std::make_shared<APSolution>(*sol_[xi])});
    if (priority) queue_.push_front(std::make_tuple(xi, xi, 0));
    else queue_.push_back(std::make_tuple(xi, xi, 0));
}

// gsAPALMData.hpp:123-132
void APALMData::appendPoint(bool priority) {
    const double x = xi_.back();
    if (priority) queue_.push_front(std::make_tuple(x, x, 0));
    else queue_.push_back(std::make_tuple(x, x, 0));
}

// gsAPALMData.hpp:134-174
void APALMData::appendData(double time, const APSolution& s, bool priority) {
    if (!t_.empty() && !(time > t_.back())) throw std::logic_error("APALM data: time must grow");
    double xi;
    if (t_.empty()) xi = 0.0;
    else if (t_.size() == 1) xi = 1.0;
    else xi = (time - t_.back()) * (xi_.back() - xi_.front()) / (t_.back() - t_.front()) + xi_.back();
    sol_.insert({xi, std::make_shared<APSolution>(s)});
    lev_.insert({xi, 0});
    if (t_.empty()) {
        prev_.insert({xi, std::make_shared<APSolution>(*sol_[xi])});
    } else {
        prev_.insert({xi, std::make_shared<APSolution>(*sol_[xi_.back()])});
        if (priority) queue_.push_front(std::make_tuple(xi_.back(), xi, 1));
        else queue_.push_back(std::make_tuple(xi_.back(), xi, 1));
    }
    insertKnot(t_, time);
    insertKnot(xi_, xi);
    buildMap();
}

// gsAPALMData.hpp:176-196: times as knots, parameters = times mapped affinely onto [0, 1]
void APALMData::setData(const std::vector<double>& times, const std::vector<APSolution>& sols) {
    t_ = times;
    std::sort(t_.begin(), t_.end());
    xi_.resize(t_.size());
    const double a = t_.front(), b = t_.back();
    for (size_t k = 0; k < t_.size(); ++k) xi_[k] = (t_[k] - a) / (b - a);
    sol_.insert({xi_[0], std::make_shared<APSolution>(sols.at(0))});
    lev_.insert({xi_[0], 0});
    prev_.insert({xi_[0], std::make_shared<APSolution>(*sol_[xi_[0]])});
    for (size_t k = 1; k < xi_.size(); ++k) {
        sol_.insert({xi_[k], std::make_shared<APSolution>(sols.at(k))});
        lev_.insert({xi_[k], 0});
        prev_.insert({xi_[k], std::make_shared<APSolution>(*sol_[xi_[k - 1]])});
    }
}

// gsAPALMData.hpp:212-247
APALMData::Job APALMData::pop() {
    if (queue_.empty()) throw std::logic_error("APALM data: the queue is empty");
    double xilow, xiupp;
    int level;
    std::tie(xilow, xiupp, level) = queue_.front();
    queue_.pop_front();
    const double tlow = tmap_[xilow], tupp = tmap_[xiupp];
    const double dt = (xilow == xiupp && level == 0) ? dt_ : tupp - tlow;
    if (!sol_.count(xilow) || !prev_.count(xilow)) throw std::logic_error("APALM data: no start point");
    APSolution start = *sol_[xilow], prev = *prev_[xilow];
    jobs_[ID_++] = std::make_tuple(xilow, xiupp, level);
    return std::make_tuple(ID_ - 1, dt, start, prev);
}

// gsAPALMData.hpp:273-283: the solution at the upper end of the job's interval
bool APALMData::referenceByID(int ID, APSolution& out) {
    const double xiupp = std::get<1>(jobs_[ID]);
    if (!sol_.count(xiupp)) return false;
    out = *sol_[xiupp];
    return true;
}

std::pair<double, double> APALMData::jobTimes(int ID) {
    const auto& j = jobs_.at(ID);
    return {tmap_[std::get<0>(j)], tmap_[std::get<1>(j)]};
}

// gsAPALMData.hpp:285-417
void APALMData::submit(int ID, const std::vector<double>& distances, std::vector<APSolution> sols, double upper,
                       double lower) {
    if (distances.size() != sols.size() + 1) throw std::logic_error("APALM data: one more distance than solutions");
    double xilow, xiupp;
    int level;
    std::tie(xilow, xiupp, level) = jobs_[ID];
    const double tlow = tmap_[xilow], tupp = tmap_[xiupp];
    const double dxi = xiupp - xilow;
    const double Dt = tupp - tlow;   // original interval length
    std::vector<double> t(distances.size() + 1);
    t[0] = tlow;
    for (size_t k = 0; k < distances.size(); ++k) t[k + 1] = t[k] + distances[k];
    // the sub-steps (all but the last distance, which is to the reference) must cover the interval
    const double dt_tmp = std::accumulate(distances.begin(), distances.end() - 1, 0.0);
    if (!((Dt - dt_tmp) / Dt < 1e-12))
        throw std::runtime_error("APALM: the sub-steps do not cover the interval");
    const double dt = t.back() - tlow;
    const double totalError = dt - upper;
    const double lowerError = Dt - lower;
    const double upperError = totalError - lowerError;
    std::vector<double> xi(sols.size() + 2);
    xi.front() = xilow;
    xi.back() = xiupp;
    for (size_t k = 1; k + 1 < xi.size(); ++k) xi[k] = xilow + dxi * (t[k] - t.front()) / dt;
    // queue the sub-intervals whose errors exceed the tolerance
    size_t kmin = 1, kmax = xi.size();
    if (lowerError / Dt < tolerance) kmin = xi.size() - 1;
    if (upperError / Dt < tolerance) kmax = xi.size() - 1;
    for (size_t k = kmin; k < kmax; ++k)
        if (level < maxLevel) queue_.push_back(std::make_tuple(xi[k - 1], xi[k], level + 1));
    // shift the curve times from the upper end on by the extra travelled length
    // (gsKnotVector::addConstant(start, amount): every knot >= start)
    for (double& v : t_)
        if (v >= tupp) v += dt - Dt;
    for (size_t k = 1; k + 1 < t.size(); ++k) {
        insertKnot(t_, t[k]);
        insertKnot(xi_, xi[k]);
    }
    buildMap();
    for (size_t k = 1; k + 1 < xi.size(); ++k) {
        sol_[xi[k]] = std::make_shared<APSolution>(sols[k - 1]);
        lev_[xi[k]] = level;
    }
    for (size_t k = 1; k + 1 < xi.size(); ++k) prev_[xi[k]] = std::make_shared<APSolution>(*sol_[xi[k - 1]]);
}

// gsAPALMData.hpp:477-499
void APALMData::flat(std::vector<double>& t, std::vector<APSolution>& s, std::vector<int>& lv) const {
    t.clear(); s.clear(); lv.clear();
    for (const auto& kv : sol_) {
        auto it = tmap_.find(kv.first);
        t.push_back(it != tmap_.end() ? it->second : 0.0);
        s.push_back(*kv.second);
        auto jt = lev_.find(kv.first);
        lv.push_back(jt != lev_.end() ? jt->second : 0);
    }
}

// gsAPALMData.hpp:570-581: parameter <-> time maps from the two knot vectors
void APALMData::buildMap() {
    if (xi_.size() != t_.size()) throw std::logic_error("APALM data: knot vectors differ in length");
    tmap_.clear();
    ximap_.clear();
    for (size_t k = 0; k < xi_.size(); ++k) {
        tmap_.insert({xi_[k], t_[k]});
        ximap_.insert({t_[k], xi_[k]});
    }
}

// ---- gsAPALM (gsALMSolvers/gsAPALM.hpp) -------------------------------------------------------

APALM::APALM(ALMGPU& alm, const Options& opt) : alm_(alm), P_(alm.problem()) {
    // gsAPALM.hpp:64-84 and gsAPALMData.hpp:57-68
    maxIt_ = (int)opt.integer("MaxIt", 1000);
    subIntervals_ = (int)opt.integer("SubIntervals", 2);
    singularPoint_ = opt.integer("SingularPoint", 0) != 0;
    branchLengthMult_ = opt.real("BranchLengthMultiplier", 1.0);
    bifLengthMult_ = opt.real("BifLengthMultiplier", 0.1);
    dataMaxLevel_ = (int)opt.integer("MaxLevel", 5);
    dataTol_ = opt.real("Tolerance", 1e-1);
    if (subIntervals_ < 1) throw std::invalid_argument("APALM: SubIntervals must be >= 1");
    if (alm_.method() != ALMGPU::Crisfield && alm_.method() != ALMGPU::Riks)
        throw std::invalid_argument("APALM needs an arc-length method with a distance (Crisfield or Riks)");
    workers_.push_back(APWorker{&alm_, &P_, std::make_shared<DevBuf<double>>(P_.nfree)});
}

APSolution APALM::copy_of(APWorker& w, const double* d_U, double L) {
    APSolution s;
    s.U = std::make_shared<DevBuf<double>>(w.P->nfree);
    KL_CUDA(cudaMemcpyAsync(s.U->get(), d_U, sizeof(double) * w.P->nfree, cudaMemcpyDeviceToDevice, w.P->stream));
    s.L = L;
    return s;
}

APSolution APALM::copy_current(APWorker& w) { return copy_of(w, w.alm->U(), w.alm->L()); }

double APALM::distance_between(APWorker& w, const APSolution& a, const APSolution& b) {
    vec::lincomb(1.0, a.U->get(), -1.0, b.U->get(), w.tmp->get(), w.P->nfree, w.P->stream);
    return w.alm->distance(w.tmp->get(), a.L - b.L);
}

void APALM::add_worker(ALMGPU& alm, Problem& P) {
    if (P.nfree != P_.nfree) throw std::invalid_argument("APALM worker: its problem has a different number of dofs");
    if (alm.method() != alm_.method()) throw std::invalid_argument("APALM worker: a different arc-length method");
    if (&P == &P_) throw std::invalid_argument("APALM worker: it needs its own problem (its own stream and state)");
    workers_.push_back(APWorker{&alm, &P, std::make_shared<DevBuf<double>>(P.nfree)});
}

void APALM::initialize() {
    if (starts_.empty()) {
        DevBuf<double> z(P_.nfree);
        z.zero(P_.stream);
        add_start(z.get(), 0.0, alm_.length());
        KL_CUDA(cudaStreamSynchronize(P_.stream));
    }
}

void APALM::add_start(const double* d_U, double L, double dL) {
    starts_.push_back(std::make_tuple(copy_of(d_U, L), dL, false));
}

bool APALM::data_empty() const {
    for (const auto& d : data_)
        if (!d.empty()) return false;
    return true;
}

int APALM::first_nonempty_branch() const {
    int k = 0;
    while (k < (int)data_.size() && data_[k].empty()) ++k;
    return k;
}

// gsAPALM.hpp:934-1011
void APALM::initiation(const APALMData::Job& job, double startTime, double& distance, std::vector<APSolution>& sols,
                       bool& bifurcation) {
    (void)startTime;
    int ID;
    double dL;
    APSolution start, prev;
    std::tie(ID, dL, start, prev) = job;
    sols.clear();
    alm_.set_length(dL);
    alm_.set_solution(start.U->get(), start.L);
    alm_.set_previous(prev.U->get(), prev.L);
    bifurcation = false;
    for (int tries = 0;; ++tries) {
        if (tries > step_retry_limit()) throw std::runtime_error("APALM: the arc-length step keeps failing");
        const int status = alm_.step();
        if (status == ST_SUCCESS) break;
        if (status == ST_NOT_CONVERGED || status == ST_ASSEMBLY_ERROR) {
            dL /= 2;
            alm_.set_length(dL);
            alm_.set_solution(start.U->get(), start.L);
        }
    }
    if (singularPoint_) {
        alm_.compute_stability(alm_.quasi(), -1e2);
        if (alm_.stability_change() && alm_.is_bifurcation(false)) {
            alm_.compute_singular_point(start.U->get(), start.L, false, false, false);
            bifurcation = true;
        }
    }
    APSolution cur = copy_current();
    distance = distance_between(cur, start);
    sols.push_back(cur);
    if (bifurcation) {
        alm_.switch_branch();
        sols.push_back(copy_current());
    }
}

// gsAPALM.hpp:1013-1170
void APALM::correction(APWorker& w, const APALMData::Job& job, std::pair<double, double> interval,
                       const APSolution& reference, std::vector<double>& distances,
                       std::vector<APSolution>& stepSolutions, double& upper, double& lower) {
    ALMGPU& alm = *w.alm;
    int N = subIntervals_;
    stepSolutions.assign(N, APSolution());
    distances.assign(N + 1, 0.0);
    int ID;
    double dL0;
    APSolution start, prev;
    std::tie(ID, dL0, start, prev) = job;
    (void)interval;
    APSolution old = start;
    const APSolution ori = start;
    dL0 /= N;
    double dL = dL0, dL_rem = 0.0;
    bool bisected = false;
    alm.set_length(dL);
    alm.set_solution(start.U->get(), start.L);
    alm.set_previous(prev.U->get(), prev.L);
    int tries = 0;
    for (int k = 0; k != N; ++k) {
        const int status = alm.step();
        if (status == ST_NOT_CONVERGED || status == ST_ASSEMBLY_ERROR) {
            if (++tries > step_retry_limit()) throw std::runtime_error("APALM: the arc-length step keeps failing");
            dL /= 2.0;
            dL_rem += dL;   // the remainder of the interval
            alm.set_length(dL);
            alm.set_solution(old.U->get(), old.L);
            bisected = true;
            k -= 1;
            continue;
        }
        stepSolutions[k] = copy_current(w);
        distances[k] = distance_between(w, stepSolutions[k], old);
        old = stepSolutions[k];
        if (!bisected) {
            dL = dL0;
        } else {
            // the interval was halved: the next sub-step covers the remainder, one more sub-step
            dL = dL_rem;
            ++N;
            stepSolutions.resize(N);
            distances.resize(N + 1);
        }
        alm.set_length(dL);
        dL_rem = 0.0;
        bisected = false;
    }
    APSolution cur = copy_current(w);
    distances.back() = distance_between(w, reference, cur);
    upper = distance_between(w, reference, ori);
    lower = distance_between(w, stepSolutions.back(), ori);
    KL_CUDA(cudaStreamSynchronize(w.P->stream));
}

// gsAPALM.hpp:122-220
void APALM::serial_solve(int nsteps) {
    if (starts_.empty()) throw std::logic_error("APALM: no start point (call initialize)");
    while (!starts_.empty()) {
        bool finished = false;
        std::vector<APSolution> sols;
        std::vector<double> times;
        std::vector<int> levels;
        APSolution start0;
        double dL, dL0;
        bool bisected;
        std::tie(start0, dL, bisected) = starts_.front();
        starts_.pop_front();
        dL0 = dL;
        APSolution old = start0, prev = start0;
        double s = 0.0;
        if (bisected) {
            dL *= bifLengthMult_;
        } else {
            sols.push_back(start0);
            times.push_back(s);
            levels.push_back(0);
        }
        std::vector<APSolution> tmp;
        for (int k = 1; k < nsteps && !finished; ++k) {
            APALMData::Job job = std::make_tuple(k, dL, old, prev);
            double distance = 0.0;
            initiation(job, s, distance, tmp, finished);
            s += distance;
            sols.push_back(tmp[0]);
            times.push_back(s);
            levels.push_back(0);
            prev = old;
            old = tmp[0];
            if (finished) starts_.push_back(std::make_tuple(tmp[1], dL0 * branchLengthMult_, true));
            dL = dL0;
        }
        APALMData data;
        data.maxLevel = dataMaxLevel_;
        data.tolerance = dataTol_;
        data.setData(times, sols);
        data.init();
        data_.push_back(data);
        sols_.push_back(sols);
        times_.push_back(times);
        levels_.push_back(levels);
    }
}

// gsAPALM.hpp:430-472
void APALM::parallel_solve() {
    if (workers_.size() > 1) return parallel_solve_workers();
    int it = 0;
    while (!data_empty() && it < maxIt_) {
        const int b = first_nonempty_branch();
        APALMData::Job job = data_[b].pop();
        const int ID = std::get<0>(job);
        APSolution reference;
        if (!data_[b].referenceByID(ID, reference)) throw std::logic_error("APALM: reference not found");
        std::vector<double> distances;
        std::vector<APSolution> stepSolutions;
        double upper = 0.0, lower = 0.0;
        correction(workers_[0], job, data_[b].jobTimes(ID), reference, distances, stepSolutions, upper, lower);
        data_[b].submit(ID, distances, stepSolutions, upper, lower);
        data_[b].finishJob(ID);
        ++it;
    }
    finalize();
}

// gsAPALM.hpp:276-378 with W workers: hand a job to every idle worker (queue order, workers in
// FIFO order), then take the oldest job handed out, submit it, return its worker to the pool and
// hand out jobs again.  The jobs of the busy workers run concurrently, one host thread each.
void APALM::parallel_solve_workers() {
    struct Flight {
        int b, ID, w;
        std::vector<double> distances;
        std::vector<APSolution> sols;
        double upper = 0.0, lower = 0.0;
        std::future<void> done;
    };
    std::deque<int> idle;
    for (int w = 0; w < (int)workers_.size(); ++w) idle.push_back(w);
    std::deque<std::unique_ptr<Flight>> flights;
    int it = 0;
    auto dispatch = [&] {
        while (!data_empty() && it < maxIt_ && !idle.empty()) {
            const int b = first_nonempty_branch();
            APALMData::Job job = data_[b].pop();
            auto f = std::make_unique<Flight>();
            f->b = b;
            f->ID = std::get<0>(job);
            f->w = idle.front();
            idle.pop_front();
            APSolution reference;
            if (!data_[b].referenceByID(f->ID, reference)) throw std::logic_error("APALM: reference not found");
            const std::pair<double, double> interval = data_[b].jobTimes(f->ID);
            // the job's start / previous / reference buffers are complete before another stream reads them
            for (auto& wk : workers_) KL_CUDA(cudaStreamSynchronize(wk.P->stream));
            Flight* fp = f.get();
            fp->done = std::async(std::launch::async, [this, fp, job, interval, reference] {
                correction(workers_[fp->w], job, interval, reference, fp->distances, fp->sols, fp->upper, fp->lower);
            });
            flights.push_back(std::move(f));
            ++it;
        }
    };
    dispatch();
    while (!flights.empty()) {
        std::unique_ptr<Flight> f = std::move(flights.front());
        flights.pop_front();
        f->done.get();   // rethrows a worker's failure
        data_[f->b].submit(f->ID, f->distances, f->sols, f->upper, f->lower);
        data_[f->b].finishJob(f->ID);
        idle.push_back(f->w);
        dispatch();
    }
    finalize();
}

// gsAPALM.hpp:822-932
void APALM::solve(int nsteps) {
    std::vector<int> K;
    while (!starts_.empty()) {
        APSolution start0;
        double dL;
        bool bisected;
        std::tie(start0, dL, bisected) = starts_.front();
        starts_.pop_front();
        APALMData data;
        data.maxLevel = dataMaxLevel_;
        data.tolerance = dataTol_;
        data_.push_back(data);
        K.push_back(1);
        data_.back().addStartPoint(0.0, start0);
        data_.back().setLength(dL);
    }
    int it = 0;
    while (!data_empty() && it < maxIt_) {
        int b = first_nonempty_branch();
        APALMData::Job job = data_[b].pop();
        const int ID = std::get<0>(job);
        const int level = data_[b].jobLevel(ID);
        if (level == 0) {
            const double startTime = data_[b].jobStartTime(ID);
            double distance = 0.0;
            std::vector<APSolution> sols;
            bool bifurcation = false;
            initiation(job, startTime, distance, sols, bifurcation);
            data_[b].appendData(startTime + distance, sols[0], false);
            data_[b].finishJob(ID);
            if (K[b]++ < nsteps - 1) {
                if (!bifurcation) {
                    data_[b].appendPoint(true);
                    if (b != 0 && ID == 0) data_[b].setLength(data_[b].getLength() / bifLengthMult_);
                } else {
                    APALMData nd;
                    nd.maxLevel = dataMaxLevel_;
                    nd.tolerance = dataTol_;
                    data_.push_back(nd);
                    K.push_back(1);
                    data_.back().addStartPoint(0.0, sols[1], true);
                    data_.back().setLength(alm_.length() * branchLengthMult_ * bifLengthMult_);
                }
            }
        } else {
            APSolution reference;
            if (!data_[b].referenceByID(ID, reference)) throw std::logic_error("APALM: reference not found");
            std::vector<double> distances;
            std::vector<APSolution> stepSolutions;
            double upper = 0.0, lower = 0.0;
            correction(workers_[0], job, data_[b].jobTimes(ID), reference, distances, stepSolutions, upper, lower);
            data_[b].submit(ID, distances, stepSolutions, upper, lower);
            data_[b].finishJob(ID);
            ++it;
        }
    }
    finalize();
}

// gsAPALM.hpp:474-504
void APALM::finalize() {
    const size_t nb = data_.size();
    sols_.assign(nb, {});
    times_.assign(nb, {});
    levels_.assign(nb, {});
    for (size_t b = 0; b < nb; ++b) data_[b].flat(times_[b], sols_[b], levels_[b]);
}

}  // namespace klsa
