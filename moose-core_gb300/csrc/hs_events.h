// hs_events.h -- the host side of synaptic events queued at run time
// (SimpleSynHandler::addSpike, synapse/SimpleSynHandler.cpp:86-90).
//
// A solver's queue is a CSR over its SynChans: SynChan k's events are
// [ptr[k], ptr[k+1]) sorted by time, of which those before the device cursor
// cur[k] are delivered.  mergeEventQueue builds the next queue: per SynChan
// the undelivered events merged with the pushed ones in time order, queued
// events first on equal times and pushed ones in push order -- the order in
// which SimpleSynHandler::vProcess pops its heap for distinct times.
// Delivered events are dropped.  No CUDA: the merge is tested on the host.
#pragma once

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <vector>

namespace hsg {

// `out` receives 2S+1 bounds/cursors: out[k] = start of SynChan k (k <= S,
// out[S] = the event count), out[S+1+k] = its cursor (= out[k]).  Returns
// false, leaving the outputs untouched, if the new queue would not fit
// 32-bit indices.  `cur` is clamped into each SynChan's range.
inline bool mergeEventQueue(uint32_t S, const std::vector<uint32_t>& ptr, const std::vector<double>& time,
                            const std::vector<double>& weight, std::vector<uint32_t> cur,
                            const std::vector<uint32_t>& pushSyn, const std::vector<double>& pushTime,
                            const std::vector<double>& pushW, std::vector<uint32_t>& out,
                            std::vector<double>& outTime, std::vector<double>& outW) {
    const size_t n = pushSyn.size();
    size_t total = n;
    for (uint32_t k = 0; k < S; ++k) {
        cur[k] = std::min(std::max(cur[k], ptr[k]), ptr[k + 1]);
        total += ptr[k + 1] - cur[k];
    }
    if (total > 0xffffffffull) return false;
    std::vector<uint32_t> ord(n);
    for (size_t i = 0; i < n; ++i) ord[i] = (uint32_t)i;
    std::stable_sort(ord.begin(), ord.end(), [&](uint32_t a, uint32_t b) {
        if (pushSyn[a] != pushSyn[b]) return pushSyn[a] < pushSyn[b];
        return pushTime[a] < pushTime[b];
    });
    std::vector<uint32_t> nptr(2 * (size_t)S + 1);
    std::vector<double> nt, nw;
    nt.reserve(total);
    nw.reserve(total);
    size_t p = 0;
    for (uint32_t k = 0; k < S; ++k) {
        nptr[k] = (uint32_t)nt.size();
        uint32_t a = cur[k];
        const uint32_t aEnd = ptr[k + 1];
        size_t pe = p;
        while (pe < n && pushSyn[ord[pe]] == k) ++pe;
        while (a < aEnd || p < pe) {
            if (p == pe || (a < aEnd && time[a] <= pushTime[ord[p]])) {
                nt.push_back(time[a]);
                nw.push_back(weight[a]);
                ++a;
            } else {
                nt.push_back(pushTime[ord[p]]);
                nw.push_back(pushW[ord[p]]);
                ++p;
            }
        }
    }
    nptr[S] = (uint32_t)nt.size();
    for (uint32_t k = 0; k < S; ++k) nptr[S + 1 + k] = nptr[k];
    out.swap(nptr);
    outTime.swap(nt);
    outW.swap(nw);
    return true;
}

}  // namespace hsg
