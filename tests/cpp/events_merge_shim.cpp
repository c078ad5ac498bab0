// Host shim over hsg::mergeEventQueue (moose-core_gb300/csrc/hs_events.h)
// for tests/test_events_merge.py: flat arrays in, flat arrays out.
#include <cstdint>
#include <cstring>
#include <vector>

#include "hs_events.h"

extern "C" int merge_events(uint32_t S, const uint32_t* ptr, const double* time, const double* weight,
                            const uint32_t* cur, uint32_t nPush, const uint32_t* pushSyn,
                            const double* pushTime, const double* pushW, uint32_t cap, uint32_t* outPtr,
                            double* outTime, double* outW, uint32_t* outN) {
    std::vector<uint32_t> p(ptr, ptr + S + 1), c(cur, cur + S), ps(pushSyn, pushSyn + nPush), op;
    std::vector<double> t(time, time + p[S]), w(weight, weight + p[S]), pt(pushTime, pushTime + nPush),
        pw(pushW, pushW + nPush), ot, ow;
    if (!hsg::mergeEventQueue(S, p, t, w, c, ps, pt, pw, op, ot, ow)) return 1;
    *outN = (uint32_t)ot.size();
    if (ot.size() > cap) return 2;
    std::memcpy(outPtr, op.data(), op.size() * sizeof(uint32_t));
    std::memcpy(outTime, ot.data(), ot.size() * sizeof(double));
    std::memcpy(outW, ow.data(), ow.size() * sizeof(double));
    return 0;
}
