// Scripted run of klsa::APALMData (the native gsAPALMData restatement, host code of the built
// library) with placeholder solutions that carry only their load factor.  Prints every job and
// the final flat solution so that tests/test_cpp_apalm_data.py can compare it line by line with
// the oracle's independent restatement.  No device memory is touched.
#include <cstdio>
#include <vector>

#include "apalm.h"

using klsa::APALMData;
using klsa::APSolution;

static APSolution sol(double L) {
    APSolution s;
    s.L = L;
    return s;
}

static void flat(const APALMData& d, const char* tag) {
    std::vector<double> t;
    std::vector<APSolution> s;
    std::vector<int> lv;
    d.flat(t, s, lv);
    for (size_t k = 0; k < t.size(); ++k) std::printf("%s %.17g %.17g %d\n", tag, t[k], s[k].L, lv[k]);
}

int main() {
    // corrections on a coarse path of four points (gsAPALMData::setData / init / pop / submit)
    APALMData d;
    d.maxLevel = 2;
    d.tolerance = 0.05;
    d.setData({0.0, 1.0, 2.0, 3.0}, {sol(0.0), sol(1.0), sol(2.0), sol(3.0)});
    d.init();
    for (int it = 0; it < 12 && !d.empty(); ++it) {
        APALMData::Job job = d.pop();
        const int ID = std::get<0>(job);
        const double dt = std::get<1>(job);
        APSolution ref;
        if (!d.referenceByID(ID, ref)) return 1;
        const int level = d.jobLevel(ID);
        std::printf("job %d %.17g %.17g %.17g %.17g %d\n", ID, dt, std::get<2>(job).L, std::get<3>(job).L, ref.L, level);
        // two sub-steps covering the interval, a distance to the reference that shrinks with the level
        std::vector<double> dist = {0.5 * dt, 0.5 * dt, 0.2 * dt / (1 + level) * (1 + 0.1 * ID)};
        std::vector<APSolution> sols = {sol(100.0 + 10 * ID), sol(101.0 + 10 * ID)};
        const double upper = dt * (1.0 + 0.03 * ID), lower = dt * (1.0 - 0.04 * (ID % 3));
        d.submit(ID, dist, sols, upper, lower);
        d.finishJob(ID);
    }
    flat(d, "flat");

    // a branch grown point by point (addStartPoint / appendData / appendPoint, the solve() path)
    APALMData b;
    b.maxLevel = 1;
    b.tolerance = 0.05;
    b.addStartPoint(0.0, sol(0.0));
    b.setLength(0.25);
    double t = 0.0;
    for (int it = 0; it < 10 && !b.empty(); ++it) {
        APALMData::Job job = b.pop();
        const int ID = std::get<0>(job);
        const double dt = std::get<1>(job);
        const int level = b.jobLevel(ID);
        std::printf("bjob %d %.17g %.17g %d\n", ID, dt, std::get<2>(job).L, level);
        if (level == 0) {
            const double start = b.jobStartTime(ID);
            t = start + dt * (1.0 + 0.01 * ID);
            b.appendData(t, sol(1000.0 + ID));
            b.finishJob(ID);
            if (it < 4) b.appendPoint(true);
        } else {
            APSolution ref;
            if (!b.referenceByID(ID, ref)) return 1;
            std::vector<double> dist = {0.5 * dt, 0.5 * dt, 0.3 * dt};
            b.submit(ID, dist, {sol(2000.0 + ID), sol(2001.0 + ID)}, dt * 1.05, dt * 0.9);
            b.finishJob(ID);
        }
    }
    flat(b, "bflat");
    return 0;
}
