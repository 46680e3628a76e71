"""FP64 CPU restatement of gsAPALM and gsAPALMData (TEST INFRASTRUCTURE ONLY).

Only tests/ import this module, as the checker of the device-side APALM.  It drives an oracle
arc-length object (oracle.ALMCrisfield / ALMRiks) with the reference's single-process schedule:

  APALMData      gsALMSolvers/gsAPALMData.hpp:20-581 (knot vectors of curve time t and parameter
                 xi, solutions / previous solutions / levels keyed by xi, job queue, submit)
  APALM          gsALMSolvers/gsAPALM.hpp:64-220 (options, initialize, serialSolve),
                 :430-504 (parallelSolve without workers, _finalize), :822-932 (solve without
                 workers), :934-1170 (_initiation, _correction)

gsKnotVector (gismo core, not in the reference tree) is stood in for by a sorted list with
repeats; addConstant(start, amount) adds amount to every knot >= start.
"""
from __future__ import annotations

import bisect
from collections import deque

import numpy as np

SUCCESS, NOT_CONVERGED, ASSEMBLY_ERROR = 0, 1, 2


class APALMData:
    def __init__(self, max_level=5, tolerance=1e-1):
        self.max_level, self.tolerance = max_level, tolerance
        self.t, self.xi = [], []
        self.sol, self.prev, self.lev = {}, {}, {}
        self.tmap, self.ximap = {}, {}
        self.queue = deque()
        self.jobs = {}
        self.ID = 0
        self.dt = 1.0

    def _build_map(self):
        self.tmap, self.ximap = {}, {}
        for x, t in zip(self.xi, self.t):
            self.tmap.setdefault(x, t)
            self.ximap.setdefault(t, x)

    def init(self):
        self.queue = deque((self.xi[k], self.xi[k + 1], 1) for k in range(len(self.xi) - 1))
        self._build_map()

    def add_start_point(self, time, s, priority=False):
        bisect.insort(self.t, time)
        bisect.insort(self.xi, 0.0)
        self.sol.setdefault(0.0, s)
        self.lev.setdefault(0.0, 0)
        self.prev.setdefault(0.0, self.sol[0.0])
        (self.queue.appendleft if priority else self.queue.append)((0.0, 0.0, 0))

    def append_point(self, priority=False):
        x = self.xi[-1]
        (self.queue.appendleft if priority else self.queue.append)((x, x, 0))

    def append_data(self, time, s, priority=False):
        if not self.t:
            x = 0.0
        elif len(self.t) == 1:
            x = 1.0
        else:
            x = (time - self.t[-1]) * (self.xi[-1] - self.xi[0]) / (self.t[-1] - self.t[0]) + self.xi[-1]
        self.sol.setdefault(x, s)
        self.lev.setdefault(x, 0)
        if not self.t:
            self.prev.setdefault(x, self.sol[x])
        else:
            self.prev.setdefault(x, self.sol[self.xi[-1]])
            (self.queue.appendleft if priority else self.queue.append)((self.xi[-1], x, 1))
        bisect.insort(self.t, time)
        bisect.insort(self.xi, x)
        self._build_map()

    def set_data(self, times, sols):
        self.t = sorted(times)
        a, b = self.t[0], self.t[-1]
        self.xi = [(v - a) / (b - a) for v in self.t]
        self.sol.setdefault(self.xi[0], sols[0])
        self.lev.setdefault(self.xi[0], 0)
        self.prev.setdefault(self.xi[0], sols[0])
        for k in range(1, len(self.xi)):
            self.sol.setdefault(self.xi[k], sols[k])
            self.lev.setdefault(self.xi[k], 0)
            self.prev.setdefault(self.xi[k], self.sol[self.xi[k - 1]])

    def empty(self):
        return not self.queue

    def pop(self):
        xilow, xiupp, level = self.queue.popleft()
        tlow, tupp = self.tmap.get(xilow, 0.0), self.tmap.get(xiupp, 0.0)
        dt = self.dt if (xilow == xiupp and level == 0) else tupp - tlow
        start, prev = self.sol[xilow], self.prev[xilow]
        self.jobs[self.ID] = (xilow, xiupp, level)
        self.ID += 1
        return self.ID - 1, dt, start, prev

    def reference(self, ID):
        return self.sol.get(self.jobs[ID][1])

    def job_times(self, ID):
        xl, xu, _ = self.jobs[ID]
        return self.tmap.get(xl, 0.0), self.tmap.get(xu, 0.0)

    def job_level(self, ID):
        return self.jobs[ID][2]

    def job_start_time(self, ID):
        return self.tmap.get(self.jobs[ID][0], 0.0)

    def finish_job(self, ID):
        del self.jobs[ID]

    def submit(self, ID, distances, sols, upper, lower):
        assert len(distances) == len(sols) + 1
        xilow, xiupp, level = self.jobs[ID]
        tlow, tupp = self.tmap[xilow], self.tmap[xiupp]
        dxi, Dt = xiupp - xilow, tupp - tlow
        t = [tlow]
        for d in distances:
            t.append(t[-1] + d)
        covered = 0.0
        for d in distances[:-1]:
            covered += d
        if not (Dt - covered) / Dt < 1e-12:
            raise RuntimeError("sub-steps do not cover the interval")
        dt = t[-1] - tlow
        total = dt - upper
        lower_err = Dt - lower
        upper_err = total - lower_err
        xi = [xilow] + [xilow + dxi * (t[k] - t[0]) / dt for k in range(1, len(sols) + 1)] + [xiupp]
        kmin, kmax = 1, len(xi)
        if lower_err / Dt < self.tolerance:
            kmin = len(xi) - 1
        if upper_err / Dt < self.tolerance:
            kmax = len(xi) - 1
        for k in range(kmin, kmax):
            if level < self.max_level:
                self.queue.append((xi[k - 1], xi[k], level + 1))
        self.t = [v + (dt - Dt) if v >= tupp else v for v in self.t]
        for k in range(1, len(t) - 1):
            bisect.insort(self.t, t[k])
            bisect.insort(self.xi, xi[k])
        self._build_map()
        for k in range(1, len(xi) - 1):
            self.sol[xi[k]] = sols[k - 1]
            self.lev[xi[k]] = level
        for k in range(1, len(xi) - 1):
            self.prev[xi[k]] = self.sol[xi[k - 1]]

    def flat(self):
        keys = sorted(self.sol)
        return ([self.tmap.get(x, 0.0) for x in keys], [self.sol[x] for x in keys], [self.lev.get(x, 0) for x in keys])


class APALM:
    def __init__(self, alm, options=None):
        o = dict(MaxIt=1000, SubIntervals=2, SingularPoint=False, BranchLengthMultiplier=1.0,
                 BifLengthMultiplier=0.1, MaxLevel=5, Tolerance=1e-1)
        o.update(options or {})
        self.alm, self.o = alm, o
        self.workers = [alm]
        self.starts = deque()
        self.data = []
        self.solutions, self.times, self.levels = [], [], []

    def _new_data(self):
        return APALMData(int(self.o["MaxLevel"]), float(self.o["Tolerance"]))

    def initialize(self):
        if not self.starts:
            self.starts.append(((np.zeros(self.alm.numDof), 0.0), self.alm.arcLength, False))

    def _step_until(self, reset, halve):
        for _ in range(61):
            st = self.alm.step()
            if st == SUCCESS:
                return
            if st in (NOT_CONVERGED, ASSEMBLY_ERROR):
                halve()
                reset()
        raise RuntimeError("arc-length step keeps failing")

    def _initiation(self, job):
        _, dL, start, prev = job
        a = self.alm
        a.set_length(dL)
        a.set_solution(start[0], start[1])
        a.set_previous(prev[0], prev[1])
        state = {"dL": dL}

        def halve():
            state["dL"] /= 2
            a.set_length(state["dL"])

        self._step_until(lambda: a.set_solution(start[0], start[1]), halve)
        bif = False
        if self.o["SingularPoint"]:
            a.compute_stability(bool(a.opts["Quasi"]))
            if a.stability_change() and a.is_bifurcation(False):
                a.compute_singular_point(start[0], start[1], False, False, False)
                bif = True
        cur = (a.U.copy(), a.L)
        dist = a.distance(cur[0] - start[0], cur[1] - start[1])
        sols = [cur]
        if bif:
            a.switch_branch()
            sols.append((a.U.copy(), a.L))
        return dist, sols, bif

    def _correction(self, job, reference, alm=None):
        a = self.alm if alm is None else alm
        N = int(self.o["SubIntervals"])
        _, dL0, start, prev = job
        dL0 = dL0 / N
        dL, rem, bisected = dL0, 0.0, False
        a.set_length(dL)
        a.set_solution(start[0], start[1])
        a.set_previous(prev[0], prev[1])
        old, ori = start, start
        steps, dists = [], []
        tries = 0
        while len(steps) < N:
            st = a.step()
            if st in (NOT_CONVERGED, ASSEMBLY_ERROR):
                tries += 1
                if tries > 60:
                    raise RuntimeError("arc-length step keeps failing")
                dL /= 2.0
                rem += dL
                a.set_length(dL)
                a.set_solution(old[0], old[1])
                bisected = True
                continue
            cur = (a.U.copy(), a.L)
            steps.append(cur)
            dists.append(a.distance(cur[0] - old[0], cur[1] - old[1]))
            old = cur
            if not bisected:
                dL = dL0
            else:
                dL = rem
                N += 1
            a.set_length(dL)
            rem, bisected = 0.0, False
        cur = (a.U.copy(), a.L)
        dists.append(a.distance(reference[0] - cur[0], reference[1] - cur[1]))
        upper = a.distance(reference[0] - ori[0], reference[1] - ori[1])
        lower = a.distance(steps[-1][0] - ori[0], steps[-1][1] - ori[1])
        return dists, steps, upper, lower

    def serial_solve(self, nsteps=10):
        while self.starts:
            (U0, L0), dL, bisected = self.starts.popleft()
            dL0 = dL
            old = prev = (U0, L0)
            s = 0.0
            sols, times, levels = [], [], []
            if bisected:
                dL *= self.o["BifLengthMultiplier"]
            else:
                sols.append((U0, L0)); times.append(s); levels.append(0)
            k, finished = 1, False
            while k < nsteps and not finished:
                dist, tmp, finished = self._initiation((k, dL, old, prev))
                s += dist
                sols.append(tmp[0]); times.append(s); levels.append(0)
                prev, old = old, tmp[0]
                if finished:
                    self.starts.append((tmp[1], dL0 * self.o["BranchLengthMultiplier"], True))
                dL = dL0
                k += 1
            d = self._new_data()
            d.set_data(times, sols)
            d.init()
            self.data.append(d)
            self.solutions.append(sols); self.times.append(times); self.levels.append(levels)

    def _first_nonempty(self):
        k = 0
        while k < len(self.data) and self.data[k].empty():
            k += 1
        return k

    def _any_jobs(self):
        return any(not d.empty() for d in self.data)

    def _correct(self, b, job=None):
        job = self.data[b].pop() if job is None else job
        ID = job[0]
        ref = self.data[b].reference(ID)
        dists, steps, upper, lower = self._correction(job, ref)
        self.data[b].submit(ID, dists, steps, upper, lower)
        self.data[b].finish_job(ID)

    def add_worker(self, alm):
        """Another solver for parallel_solve (an MPI worker of the reference)."""
        self.workers.append(alm)

    def parallel_solve(self):
        if len(self.workers) > 1:
            return self._parallel_solve_workers()
        it = 0
        while self._any_jobs() and it < self.o["MaxIt"]:
            self._correct(self._first_nonempty())
            it += 1
        self._finalize()

    def _parallel_solve_workers(self):
        """gsAPALM.hpp:276-378: hand a job to every idle worker (queue order, workers FIFO), then
        take the oldest job handed out, submit it, return its worker and hand out jobs again.
        A job's correction depends only on the job and its worker, so it is computed when it is
        handed out and submitted in turn."""
        idle = deque(range(len(self.workers)))
        flights = deque()
        it = 0

        def dispatch():
            nonlocal it
            while self._any_jobs() and it < self.o["MaxIt"] and idle:
                b = self._first_nonempty()
                job = self.data[b].pop()
                ID = job[0]
                w = idle.popleft()
                res = self._correction(job, self.data[b].reference(ID), self.workers[w])
                flights.append((b, ID, w, res))
                it += 1

        dispatch()
        while flights:
            b, ID, w, res = flights.popleft()
            self.data[b].submit(ID, *res)
            self.data[b].finish_job(ID)
            idle.append(w)
            dispatch()
        self._finalize()

    def solve(self, nsteps=10):
        K = []
        while self.starts:
            (U0, L0), dL, _ = self.starts.popleft()
            d = self._new_data()
            d.add_start_point(0.0, (U0, L0))
            d.dt = dL
            self.data.append(d)
            K.append(1)
        it = 0
        while self._any_jobs() and it < self.o["MaxIt"]:
            b = self._first_nonempty()
            d = self.data[b]
            job = d.pop()
            ID = job[0]
            if d.job_level(ID) == 0:
                t0 = d.job_start_time(ID)
                dist, sols, bif = self._initiation(job)
                d.append_data(t0 + dist, sols[0], False)
                d.finish_job(ID)
                kb = K[b]
                K[b] += 1
                if kb < nsteps - 1:
                    if not bif:
                        d.append_point(True)
                        if b != 0 and ID == 0:
                            d.dt = d.dt / self.o["BifLengthMultiplier"]
                    else:
                        nd = self._new_data()
                        self.data.append(nd)
                        K.append(1)
                        nd.add_start_point(0.0, sols[1], True)
                        nd.dt = self.alm.arcLength * self.o["BranchLengthMultiplier"] * self.o["BifLengthMultiplier"]
            else:
                self._correct(b, job)
                it += 1
        self._finalize()

    def _finalize(self):
        self.solutions, self.times, self.levels = [], [], []
        for d in self.data:
            t, s, lv = d.flat()
            self.times.append(t); self.solutions.append(s); self.levels.append(lv)
