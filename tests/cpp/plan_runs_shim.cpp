// Host shim over the elimination plan (moose-core_gb300/csrc/hs_plan.cpp)
// for tests/test_plan_runs.py.  It runs the two sweeps of hs_fp64.cu's
// eliminateWarp on the host, once through the general level programs and
// once with the cable runs (CellPlan::fRun/bRun) walked the way
// forwardCableRun/backwardCableRun walk them, on the same seeded matrix,
// and reports whether M, VMid and V agree bit for bit.
#include <cstdint>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "hs_plan.h"

using namespace hsg;

namespace {

void general(const CellPlan& P, std::vector<double>& M, std::vector<double>& VMid, std::vector<double>& V) {
    const uint32_t N = P.N;
    for (size_t l = 0; l + 1 < P.fLevelPtr.size(); ++l)
        for (uint32_t k = P.fLevelPtr[l]; k < P.fLevelPtr[l + 1]; ++k)
            for (uint32_t o = P.fOpPtr[k]; o < P.fOpPtr[k + 1]; ++o) {
                const FwdOp& op = P.fOps[o];
                M[op.t] -= M[op.l] / M[op.p] * M[op.a];
            }
    for (size_t l = 0; l + 1 < P.bLevelPtr.size(); ++l)
        for (uint32_t k = P.bLevelPtr[l]; k < P.bLevelPtr[l + 1]; ++k) {
            const uint32_t i = P.bRows[k];
            double v = M[N + i];
            for (uint32_t t = P.bTermPtr[k]; t < P.bTermPtr[k + 1]; ++t) v -= M[P.bTerms[t].coef] * VMid[P.bTerms[t].src];
            v /= M[i];
            VMid[i] = v;
            V[i] = 2 * v - V[i];
        }
}

void withRuns(const CellPlan& P, std::vector<double>& M, std::vector<double>& VMid, std::vector<double>& V,
              uint32_t& fRows, uint32_t& bRows) {
    const uint32_t N = P.N, offBase = 2 * N + P.H;
    fRows = bRows = 0;
    for (size_t l = 0; l + 1 < P.fLevelPtr.size(); ++l) {
        if (const uint32_t run = P.fRun[l]) {
            fRows += run;
            uint32_t r = P.fRunRow[l];
            double d = M[r - 1], rhs = M[N + r - 1];
            for (uint32_t i = 0; i < run; ++i, ++r) {
                const double o = M[offBase + r - 1];
                const double q = o / d;
                d = M[r] - q * o;
                rhs = M[N + r] - q * rhs;
                M[r] = d;
                M[N + r] = rhs;
            }
            l += run - 1;
            continue;
        }
        for (uint32_t k = P.fLevelPtr[l]; k < P.fLevelPtr[l + 1]; ++k) {
            int32_t ql = -1, qp = -1;
            double q = 0.0;
            for (uint32_t o = P.fOpPtr[k]; o < P.fOpPtr[k + 1]; ++o) {
                const FwdOp& op = P.fOps[o];
                if (op.l != ql || op.p != qp) {
                    q = M[op.l] / M[op.p];
                    ql = op.l;
                    qp = op.p;
                }
                M[op.t] -= q * M[op.a];
                if (op.t == ql || op.t == qp) ql = -1;
            }
        }
    }
    for (size_t l = 0; l + 1 < P.bLevelPtr.size(); ++l) {
        if (const uint32_t run = P.bRun[l]) {
            bRows += run;
            uint32_t i = P.bRunRow[l];
            double vNext = VMid[i + 1];
            for (uint32_t j = 0; j < run; ++j, --i) {
                double v = M[N + i];
                v -= M[offBase + i] * vNext;
                v /= M[i];
                VMid[i] = v;
                V[i] = 2 * v - V[i];
                vNext = v;
            }
            l += run - 1;
            continue;
        }
        for (uint32_t k = P.bLevelPtr[l]; k < P.bLevelPtr[l + 1]; ++k) {
            const uint32_t i = P.bRows[k];
            double v = M[N + i];
            for (uint32_t t = P.bTermPtr[k]; t < P.bTermPtr[k + 1]; ++t) v -= M[P.bTerms[t].coef] * VMid[P.bTerms[t].src];
            v /= M[i];
            VMid[i] = v;
            V[i] = 2 * v - V[i];
        }
    }
}

}  // namespace

// stats: N, rows in forward runs, rows in backward runs, forward levels,
// backward levels.  Returns 0 if the sweeps agree, 1 if not, -1 if the plan
// could not be built.
extern "C" int plan_runs_check(const HsCellDesc* d, uint32_t seed, uint32_t* stats) {
    CellPlan P;
    std::string err;
    if (!buildPlan(*d, seed, 25e-6, P, err)) return -1;
    const uint32_t N = P.N;
    std::mt19937_64 g(seed + 1);
    std::uniform_real_distribution<double> u(0.5, 2.0);
    std::vector<double> M(3 * (size_t)N + P.H), V(N);
    for (uint32_t i = 0; i < N; ++i) {
        M[i] = 4.0 + u(g);
        M[N + i] = u(g) - 1.25;
        V[i] = u(g) * -0.06;
    }
    for (uint32_t h = 0; h < P.H; ++h) M[2 * N + h] = -u(g) * 0.3;
    for (uint32_t i = 0; i < N; ++i) M[2 * N + P.H + i] = P.off[i] != 0.0 ? -u(g) * 0.5 : 0.0;
    std::vector<double> M2 = M, V2 = V, VMid(N, 0.0), VMid2(N, 0.0);
    general(P, M, VMid, V);
    withRuns(P, M2, VMid2, V2, stats[1], stats[2]);
    stats[0] = N;
    stats[3] = (uint32_t)P.fLevelPtr.size() - 1;
    stats[4] = (uint32_t)P.bLevelPtr.size() - 1;
    const bool same = !std::memcmp(M.data(), M2.data(), M.size() * sizeof(double)) &&
                      !std::memcmp(VMid.data(), VMid2.data(), N * sizeof(double)) &&
                      !std::memcmp(V.data(), V2.data(), N * sizeof(double));
    return same ? 0 : 1;
}

// The forward sweep's waves (CellPlan::fWavePtr/fWaveOps) against the level
// programs on the same seeded matrix: the updates of each wave run last to
// first (a wave's updates touch disjoint entries, so any order gives the
// same values), then the back substitution as in general().  stats: N,
// waves (0: the plan keeps the level programs), fused updates, levels.
extern "C" int plan_waves_check(const HsCellDesc* d, uint32_t seed, uint32_t* stats) {
    CellPlan P;
    std::string err;
    if (!buildPlan(*d, seed, 25e-6, P, err)) return -1;
    const uint32_t N = P.N;
    stats[0] = N;
    stats[1] = P.fWavePtr.empty() ? 0 : (uint32_t)P.fWavePtr.size() - 1;
    stats[2] = (uint32_t)P.fWaveOps.size();
    stats[3] = (uint32_t)P.fLevelPtr.size() - 1;
    if (P.fWavePtr.empty()) return 0;
    std::mt19937_64 g(seed + 7);
    std::uniform_real_distribution<double> u(0.5, 2.0);
    std::vector<double> M(3 * (size_t)N + P.H), V(N);
    for (uint32_t i = 0; i < N; ++i) {
        M[i] = 4.0 + u(g);
        M[N + i] = u(g) - 1.25;
        V[i] = u(g) * -0.06;
    }
    for (uint32_t h = 0; h < P.H; ++h) M[2 * N + h] = -u(g) * 0.3;
    for (uint32_t i = 0; i < N; ++i) M[2 * N + P.H + i] = P.off[i] != 0.0 ? -u(g) * 0.5 : 0.0;
    std::vector<double> M2 = M, V2 = V, VMid(N, 0.0), VMid2(N, 0.0);
    general(P, M, VMid, V);
    for (size_t w = 0; w + 1 < P.fWavePtr.size(); ++w)
        for (uint32_t k = P.fWavePtr[w + 1]; k-- > P.fWavePtr[w];) {
            const FwdPair& f = P.fWaveOps[k];
            const double q = M2[f.l] / M2[f.p];
            M2[f.t1] -= q * M2[f.a1];
            if (f.t2 >= 0) M2[f.t2] -= q * M2[f.a2];
        }
    for (size_t l = 0; l + 1 < P.bLevelPtr.size(); ++l)
        for (uint32_t k = P.bLevelPtr[l]; k < P.bLevelPtr[l + 1]; ++k) {
            const uint32_t i = P.bRows[k];
            double v = M2[N + i];
            for (uint32_t t = P.bTermPtr[k]; t < P.bTermPtr[k + 1]; ++t)
                v -= M2[P.bTerms[t].coef] * VMid2[P.bTerms[t].src];
            v /= M2[i];
            VMid2[i] = v;
            V2[i] = 2 * v - V2[i];
        }
    const bool same = !std::memcmp(M.data(), M2.data(), M.size() * sizeof(double)) &&
                      !std::memcmp(VMid.data(), VMid2.data(), N * sizeof(double)) &&
                      !std::memcmp(V.data(), V2.data(), N * sizeof(double));
    return same ? 0 : 1;
}
