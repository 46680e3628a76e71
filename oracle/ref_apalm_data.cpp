// The reference's gsAPALMData (src/gsALMSolvers/gsAPALMData.hpp), compiled unchanged against the
// test-only stand-in in refshim/ (test infrastructure only; built by the Makefile target `ref`
// into _ref/).  It runs the scripted job sequence of tests/cpp/apalm_data_driver.cpp -- the same
// pops, submits and finished jobs, with placeholder solutions that carry only their load
// factor -- and prints the same lines, so that the tests can compare the product's queue
// (klsa::APALMData) and the oracle's (oracle/apalm.py) with the reference's own, line by line.
#include <cstdio>
#include <vector>

#include <gsStructuralAnalysis/src/gsALMSolvers/gsAPALMData.h>

using namespace gismo;

namespace {

struct Sol {
    double L = 0.0;
};
typedef gsAPALMData<real_t, Sol> Data;

Sol sol(double L) {
    Sol s;
    s.L = L;
    return s;
}

void flat(Data& d, const char* tag) {
    std::vector<real_t> t;
    std::vector<Sol> s;
    std::vector<index_t> lv;
    std::tie(t, s, lv) = d.getFlatSolution();
    for (size_t k = 0; k < t.size(); ++k) std::printf("%s %.17g %.17g %d\n", tag, t[k], s[k].L, (int)lv[k]);
}

int run() {
    // corrections on a coarse path of four points (setData / init / pop / submit)
    Data d;
    d.options().setInt("MaxLevel", 2);
    d.options().setReal("Tolerance", 0.05);
    d.setData({0.0, 1.0, 2.0, 3.0}, {sol(0.0), sol(1.0), sol(2.0), sol(3.0)});
    d.init();
    for (int it = 0; it < 12 && !d.empty(); ++it) {
        index_t ID;
        real_t dt;
        Sol start, prev, ref;
        std::tie(ID, dt, start, prev) = d.pop();
        if (!d.getReferenceByID(ID, ref)) return 1;
        const index_t level = d.jobLevel(ID);
        std::printf("job %d %.17g %.17g %.17g %.17g %d\n", (int)ID, dt, start.L, prev.L, ref.L, (int)level);
        std::vector<real_t> dist = {0.5 * dt, 0.5 * dt, 0.2 * dt / (1 + level) * (1 + 0.1 * ID)};
        std::vector<Sol> sols = {sol(100.0 + 10 * ID), sol(101.0 + 10 * ID)};
        d.submit(ID, dist, sols, dt * (1.0 + 0.03 * ID), dt * (1.0 - 0.04 * (ID % 3)));
        d.finishJob(ID);
    }
    flat(d, "flat");

    // a branch grown point by point (addStartPoint / appendData / appendPoint)
    Data b;
    b.options().setInt("MaxLevel", 1);
    b.options().setReal("Tolerance", 0.05);
    b.addStartPoint(0.0, sol(0.0));
    b.setLength(0.25);
    for (int it = 0; it < 10 && !b.empty(); ++it) {
        index_t ID;
        real_t dt;
        Sol start, prev;
        std::tie(ID, dt, start, prev) = b.pop();
        const index_t level = b.jobLevel(ID);
        std::printf("bjob %d %.17g %.17g %d\n", (int)ID, dt, start.L, (int)level);
        if (level == 0) {
            const real_t t = b.jobStartTime(ID) + dt * (1.0 + 0.01 * ID);
            b.appendData(t, sol(1000.0 + ID));
            b.finishJob(ID);
            if (it < 4) b.appendPoint(true);
        } else {
            Sol ref;
            if (!b.getReferenceByID(ID, ref)) return 1;
            b.submit(ID, {0.5 * dt, 0.5 * dt, 0.3 * dt}, {sol(2000.0 + ID), sol(2001.0 + ID)}, dt * 1.05, dt * 0.9);
            b.finishJob(ID);
        }
    }
    flat(b, "bflat");
    return 0;
}

}  // namespace

int main() {
    try {
        return run();
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 2;
    }
}
