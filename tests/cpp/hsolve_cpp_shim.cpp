// C entry points over the C++ HSolve mirror (moose-core_gb300/cpp/hsolve_gpu.hpp)
// for tests/test_cpp_mirror.py: the test hands a cell description to
// hsolve_cpp_run, which drives it through moose_gb300::HSolve -- field
// writes, message destinations, process and the group call -- and returns
// Vm and Ca;
// hsolve_cpp_errors checks the error behaviour, which needs no GPU.
#include <cstring>

#include "hsolve_gpu.hpp"

namespace {
void copyMsg(const char* m, char* err, uint32_t len) {
    if (!err || !len) return;
    std::strncpy(err, m, len - 1);
    err[len - 1] = 0;
}
}  // namespace

extern "C" int hsolve_cpp_run(const HsCellDesc* d, uint32_t seed, double dt, uint32_t nCompt, uint32_t nPool,
                              uint32_t nsteps, double* vmOut, double* caOut, char* err, uint32_t errlen) {
    try {
        moose_gb300::HSolve h;
        h.setDt(dt);
        h.setCaAdvance(1);
        if (!h.setTarget(*d, seed)) {
            copyMsg(hs_last_error(), err, errlen);
            return 1;
        }
        h.reinit(dt);
        h.process(nsteps / 2);
        // a field write (persists), a message (next step only), zombie fields
        h.setInject(0, 0.3e-9);
        h.addInject(nCompt - 1, 0.1e-9);
        h.setHHmodulation(0, 1.2);
        h.setHHmodulation(1, 0.0);            // ignored: a value <= 0 keeps the old one
        h.setEm(nCompt > 1 ? 1 : 0, -0.07);
        if (nPool) h.iCa(0, 1e-12);
        // the rest through the tick's group call (a group of one here)
        moose_gb300::HSolve::processGroup({&h}, nsteps - nsteps / 2);
        const std::vector<double> v = h.vm(nCompt);
        const std::vector<double> c = h.ca(nPool);
        for (uint32_t i = 0; i < nCompt; ++i) vmOut[i] = v[i];
        for (uint32_t i = 0; i < nPool; ++i) caOut[i] = c[i];
        if (h.getVm(0) != v[0] || h.steps() != nsteps) {
            copyMsg("field read and bulk read disagree", err, errlen);
            return 2;
        }
        return 0;
    } catch (const moose_gb300::Error& e) {
        copyMsg(e.what(), err, errlen);
        return 3;
    }
}

extern "C" int hsolve_cpp_errors(const HsCellDesc* d) {
    moose_gb300::HSolve h;
    if (h.getDt() != 50e-6 || h.getCaAdvance() != 1) return 1;
    h.setDt(-1.0);                            // rejected: dt stays
    if (h.getDt() != 50e-6) return 2;
    h.setCaAdvance(2);                        // rejected
    if (h.getCaAdvance() != 1) return 3;
    h.setVDiv(1000);
    if (h.getVDiv() != 1000) return 4;        // reported until setup
    h.setDt(0.0);
    if (h.setTarget(*d, 0)) return 5;         // "Must set 'dt' first"
    try {
        h.getVm(0);
        return 6;
    } catch (const moose_gb300::Error& e) {
        if (e.code() != HS_EINVAL) return 7;
    }
    try {
        h.addSpike(0, 1e-3, 1e-9);                // no solver: rejected like a field access
        return 8;
    } catch (const moose_gb300::Error& e) {
        if (e.code() != HS_EINVAL) return 9;
    }
    return 0;
}
