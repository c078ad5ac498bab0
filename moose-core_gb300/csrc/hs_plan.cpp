// hs_plan.cpp -- host-side HSolve setup (see hs_plan.h).
#include "hs_plan.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <map>
#include <numeric>
#include <set>

namespace hsg {

namespace {

struct Adj {
    // children CSR in HSolveUtils::children order: by link kind (axial,
    // distal/sphere, cylinder), increasing child index within a kind;
    // grp[k] = the first entry of kind k+1 in each node's list
    std::vector<uint32_t> off, idx;
    std::vector<uint32_t> grp;     // 2 per node: ends of the axial and distal runs
};

int linkOf(const HsCellDesc& d, uint32_t i) { return d.link ? d.link[i] : HS_LINK_AXIAL; }

Adj childrenOf(const HsCellDesc& d) {
    Adj a;
    uint32_t n = d.n_compt;
    a.off.assign(n + 1, 0);
    for (uint32_t i = 0; i < n; ++i)
        if (d.parent[i] >= 0) a.off[d.parent[i] + 1]++;
    for (uint32_t i = 0; i < n; ++i) a.off[i + 1] += a.off[i];
    a.idx.resize(a.off[n]);
    a.grp.assign(2 * (size_t)n, 0);
    std::vector<uint32_t> fill(n, 0);
    for (int kind = HS_LINK_AXIAL; kind <= HS_LINK_CYLINDER; ++kind) {
        for (uint32_t i = 0; i < n; ++i)
            if (d.parent[i] >= 0 && linkOf(d, i) == kind) {
                uint32_t p = (uint32_t)d.parent[i];
                a.idx[a.off[p] + fill[p]++] = i;
            }
        if (kind < HS_LINK_CYLINDER)
            for (uint32_t p = 0; p < n; ++p) a.grp[2 * p + kind] = a.off[p] + fill[p];
    }
    return a;
}

// HSolveUtils::adjacent (hsolve/HSolveUtils.cpp:36-45): axial targets (the
// axial children, message order), raxial targets (the parent of an axial
// link), distalOut targets (distal/sphere children), proximalOut targets
// (the parent of a SymCompartment link), cylinderOut targets (cylinder
// children), minus `exclude`.
void adjacent(const HsCellDesc& d, const Adj& ch, uint32_t c, int64_t exclude,
              std::vector<int64_t>& out) {
    const bool hasParent = d.parent[c] >= 0 && (int64_t)d.parent[c] != exclude;
    const bool axialUp = linkOf(d, c) == HS_LINK_AXIAL;
    const uint32_t e0 = ch.grp[2 * c], e1 = ch.grp[2 * c + 1];
    for (uint32_t k = ch.off[c]; k < ch.off[c + 1]; ++k) {
        if (k == e0 && hasParent && axialUp) out.push_back(d.parent[c]);
        if (k == e1 && hasParent && !axialUp) out.push_back(d.parent[c]);
        if ((int64_t)ch.idx[k] != exclude) out.push_back(ch.idx[k]);
    }
    const uint32_t end = ch.off[c + 1];
    if (hasParent && ((axialUp && e0 == end) || (!axialUp && e1 == end))) out.push_back(d.parent[c]);
}

// HSolvePassive::walkTree (hsolve/HSolvePassive.cpp:45-98): from the seed,
// follow the first neighbour to a leaf; depth-first search from that leaf
// (last neighbour first); the reversed visit order is the Hines order.
bool walkTree(const HsCellDesc& d, const Adj& ch, uint32_t seed, std::vector<uint32_t>& hinesToModel) {
    std::vector<int64_t> adj;
    adjacent(d, ch, seed, -1, adj);
    if (adj.size() > 1) {
        uint32_t guard = 0;
        while (!adj.empty()) {
            if (++guard > d.n_compt) return false;   // a cycle: not a tree
            int64_t previous = seed;
            seed = (uint32_t)adj[0];
            adj.clear();
            adjacent(d, ch, seed, previous, adj);
        }
    }
    std::vector<std::vector<int64_t>> stack(1, std::vector<int64_t>(1, seed));
    int64_t above = -1;
    std::vector<uint32_t> order;
    while (!stack.empty()) {
        std::vector<int64_t>& top = stack.back();
        if (top.empty()) {
            stack.pop_back();
            if (!stack.empty()) stack.back().pop_back();
        } else {
            if (stack.size() > 1) above = stack[stack.size() - 2].back();
            uint32_t current = (uint32_t)top.back();
            if (order.size() >= d.n_compt) return false;   // a cycle: not a tree
            order.push_back(current);
            std::vector<int64_t> next;
            adjacent(d, ch, current, above, next);
            stack.push_back(std::move(next));
        }
    }
    hinesToModel.assign(order.rbegin(), order.rend());
    return true;
}

// HHGate::lookupBoth with interpolation (biophysics/HHGate.cpp:258-283),
// used when a gate's grid differs from the merged table grid.
void gateLookupBoth(const HsGateTable& g, double v, double* A, double* B) {
    double invDx = (double)g.divs / (g.max - g.min);
    if (v <= g.min) {
        *A = g.A[0];
        *B = g.B[0];
    } else if (v >= g.max) {
        *A = g.A[g.divs];
        *B = g.B[g.divs];
    } else {
        unsigned int index = (unsigned int)((v - g.min) * invDx);
        double frac = (v - g.min - index / invDx) * invDx;
        *A = g.A[index] * (1 - frac) + g.A[index + 1] * frac;
        *B = g.B[index] * (1 - frac) + g.B[index + 1] * frac;
    }
}

// LookupTable (hsolve/RateLookup.cpp:15-54): nDivs+2 rows, last row repeated.
void initTable(Table& t, double min, double max, uint32_t nDivs, uint32_t nSpecies) {
    t.min = min;
    t.max = max;
    t.nPts = nDivs + 2;
    t.dx = (max - min) / nDivs;
    t.nCol = 2 * nSpecies;
    t.data.assign((size_t)t.nPts * t.nCol, 0.0);
}
void addColumns(Table& t, uint32_t species, const double* A, const double* B, size_t n) {
    size_t pos = 2 * species;
    for (uint32_t g = 0; g + 1 < t.nPts; ++g) {
        t.data[pos] = A[g];
        t.data[pos + 1] = B[g];
        pos += t.nCol;
    }
    t.data[pos] = A[n - 1];
    t.data[pos + 1] = B[n - 1];
}

template <class T>
bool hasN(const T* p, uint32_t n) { return n == 0 || p != nullptr; }

}  // namespace

void synchanConstants(double tau1, double tau2, double gbar, double dt, double* xc1,
                      double* xc2, double* yc1, double* yc2, double* norm) {
    *xc1 = tau1 * (1.0 - std::exp(-dt / tau1));
    *xc2 = std::exp(-dt / tau1);
    if (tau2 == 0.0) {
        *yc1 = 1.0;
        *yc2 = 0.0;
        *norm = gbar;
    } else {
        *yc1 = tau2 * (1.0 - std::exp(-dt / tau2));
        *yc2 = std::exp(-dt / tau2);
        if (tau1 == tau2) {
            *norm = gbar * std::exp(1.0) / tau1;
        } else {
            double tpeak = tau1 * tau2 * std::log(tau1 / tau2) / (tau1 - tau2);
            *norm = gbar * (tau1 - tau2) /
                    (tau1 * tau2 * (std::exp(-tpeak / tau1) - std::exp(-tpeak / tau2)));
        }
    }
}

bool buildPlan(const HsCellDesc& d, uint32_t seed, double dt, CellPlan& P, std::string& err,
               const PlanOptions& opt) {
    auto fail = [&](const std::string& m) { err = m; return false; };
    if (d.n_compt == 0) return fail("cell has no compartments");
    if (seed >= d.n_compt) return fail("seed compartment index out of range");
    if (!(dt > 0.0)) return fail("HSolve: 'dt' must be positive");
    if (!d.parent || !d.Ra || !d.Rm || !d.Cm || !d.Em || !d.initVm || !d.Vm || !d.inject)
        return fail("compartment arrays missing");
    if (!hasN(d.leak_compt, d.n_leak) || !hasN(d.gate, d.n_gate) || !hasN(d.chan_compt, d.n_chan) ||
        !hasN(d.pool_compt, d.n_pool) || !hasN(d.gate2d, d.n_gate2d) || !hasN(d.c2d_compt, d.n_chan2d) ||
        !hasN(d.syn_compt, d.n_syn) || !hasN(d.ev_syn, d.n_event) || !hasN(d.sg_compt, d.n_spikegen) ||
        !hasN(d.stim_compt, d.n_stim))
        return fail("array missing for a non-zero count");
    for (uint32_t i = 0; i < d.n_compt; ++i) {
        if (d.parent[i] >= (int32_t)d.n_compt || d.parent[i] == (int32_t)i || d.parent[i] < -1)
            return fail("bad parent index");
        if (d.link && (d.link[i] < HS_LINK_AXIAL || d.link[i] > HS_LINK_CYLINDER)) return fail("bad link kind");
        if (!(d.Ra[i] != 0.0) || !(d.Rm[i] != 0.0)) return fail("Ra and Rm must be non-zero");
    }
    for (uint32_t g = 0; g < d.n_gate; ++g)
        if (d.gate[g].divs < 1 || !d.gate[g].A || !d.gate[g].B || !(d.gate[g].max > d.gate[g].min))
            return fail("bad gate table");
    for (uint32_t g = 0; g < d.n_gate2d; ++g) {
        const HsGate2DTable& t = d.gate2d[g];
        if (t.xdivs < 1 || t.ydivs < 1 || !t.A || !t.B || !(t.xmax > t.xmin) || !(t.ymax > t.ymin))
            return fail("bad 2-D gate table");
    }

    Adj ch = childrenOf(d);
    if (!walkTree(d, ch, seed, P.modelOf)) return fail("compartment graph is not a tree");
    const uint32_t N = (uint32_t)P.modelOf.size();
    P.N = N;
    P.dtSetup = dt;
    P.hinesOf.assign(d.n_compt, -1);
    for (uint32_t i = 0; i < N; ++i) P.hinesOf[P.modelOf[i]] = i;

    // HSolvePassive::initialize (hsolve/HSolvePassive.cpp:100-165)
    std::vector<std::vector<uint32_t>> leaks(d.n_compt);
    for (uint32_t l = 0; l < d.n_leak; ++l) {
        if (d.leak_compt[l] >= d.n_compt) return fail("leakage compartment out of range");
        leaks[d.leak_compt[l]].push_back(l);
    }
    P.V0.resize(N); P.CmByDt.resize(N); P.EmByRm.resize(N);
    P.injBasal.assign(N, 0.0); P.injPresent.assign(N, 0);
    P.Ra.resize(N); P.Rm.resize(N); P.Cm.resize(N); P.Em.resize(N); P.initVm.resize(N);
    P.children.resize(N);
    for (uint32_t ic = 0; ic < N; ++ic) {
        uint32_t m = P.modelOf[ic];
        P.V0[ic] = d.Vm[m];
        double EmGmThev = d.Em[m] / d.Rm[m];
        for (uint32_t l : leaks[m]) EmGmThev += d.leak_Ek[l] * d.leak_Gk[l];
        P.CmByDt[ic] = 2.0 * d.Cm[m] / dt;
        P.EmByRm[ic] = EmGmThev;
        if (d.inject[m] != 0.0) {
            P.injPresent[ic] = 1;
            P.injBasal[ic] = d.inject[m];
        }
        // storeTree (hsolve/HSolvePassive.cpp:167-205)
        for (uint32_t k = ch.off[m]; k < ch.off[m + 1]; ++k)
            P.children[ic].push_back((uint32_t)P.hinesOf[ch.idx[k]]);
        P.Ra[ic] = d.Ra[m]; P.Rm[ic] = d.Rm[m]; P.Cm[ic] = d.Cm[m];
        P.Em[ic] = d.Em[m]; P.initVm[ic] = d.initVm[m];
    }

    // HinesMatrix::makeJunctions (hsolve/HinesMatrix.cpp:84-130)
    std::vector<double> Ga(N);
    for (uint32_t i = 0; i < N; ++i) Ga[i] = 2.0 / P.Ra[i];
    std::vector<std::vector<uint32_t>> coupled;
    for (uint32_t i = 0; i < N; ++i) {
        const std::vector<uint32_t>& c = P.children[i];
        if (c.empty()) continue;
        if (c.size() == 1) {
            int diff = (int)c[0] - (int)i;
            if (diff == 1 || diff == -1) continue;
        }
        coupled.push_back(c);
        coupled.back().push_back(i);
    }
    for (auto& g : coupled) std::sort(g.begin(), g.end());
    std::stable_sort(coupled.begin(), coupled.end(),
                     [](const std::vector<uint32_t>& a, const std::vector<uint32_t>& b) { return a[0] < b[0]; });
    struct Junction { uint32_t index, rank; };
    std::vector<Junction> junction;
    std::vector<int64_t> groupOf(N, -1);
    for (size_t g = 0; g < coupled.size(); ++g)
        for (size_t c = 0; c + 1 < coupled[g].size(); ++c) {
            junction.push_back({coupled[g][c], (uint32_t)(coupled[g].size() - c - 1)});
            groupOf[coupled[g][c]] = (int64_t)g;
        }
    std::stable_sort(junction.begin(), junction.end(),
                     [](const Junction& a, const Junction& b) { return a.index < b.index; });

    // makeMatrix (hsolve/HinesMatrix.cpp:133-223)
    P.HS2.assign(N, 0.0);
    P.off.assign(N, 0.0);
    for (uint32_t i = 0; i < N; ++i) P.HS2[i] = P.Cm[i] / (dt / 2.0) + 1.0 / P.Rm[i];
    {
        size_t jn = 0;
        for (uint32_t i = 0; i + 1 < N; ++i) {
            if (!junction.empty() && jn < junction.size() && i == junction[jn].index) {
                ++jn;
                continue;
            }
            double gi = Ga[i], gj = Ga[i + 1];
            double gij = gi * gj / (gi + gj);
            P.off[i] = -gij;
            P.HS2[i] += gij;
            P.HS2[i + 1] += gij;
        }
    }
    for (auto& g : coupled) {
        double gsum = 0.0;
        for (uint32_t c : g) gsum += Ga[c];
        for (uint32_t c : g) {
            double gi = Ga[c];
            P.HS2[c] += gi * (1.0 - gi / gsum);
        }
    }
    std::vector<int64_t> operandBase(N, -1);
    std::vector<uint32_t> hjOwner;
    for (auto& g : coupled) {
        double gsum = 0.0;
        for (uint32_t c : g) gsum += Ga[c];
        for (size_t a = 0; a + 1 < g.size(); ++a) {
            operandBase[g[a]] = (int64_t)P.HJ0.size();
            for (size_t b = a + 1; b < g.size(); ++b) {
                double gij = Ga[g[a]] * Ga[g[b]] / gsum;
                P.HJ0.push_back(-gij);
                P.HJ0.push_back(-gij);
                hjOwner.push_back(g[a]);
                hjOwner.push_back(g[a]);
            }
        }
    }
    const uint32_t H = (uint32_t)P.HJ0.size();
    P.H = H;

    // Entry numbering of the M array.
    auto DIAG = [&](uint32_t i) { return (int32_t)i; };
    auto RHS = [&](uint32_t i) { return (int32_t)(N + i); };
    auto HJE = [&](int64_t h) { return (int32_t)(2 * N + h); };
    auto OFF = [&](uint32_t i) { return (int32_t)(2 * N + H + i); };
    auto owner = [&](int32_t e) -> uint32_t {
        if (e < (int32_t)N) return (uint32_t)e;
        if (e < (int32_t)(2 * N)) return (uint32_t)(e - N);
        return hjOwner[e - 2 * N];
    };

    // Forward elimination as the reference sweeps it (HSolvePassive::
    // forwardEliminate + makeOperands), emitted as (t, l, a, pivot) updates.
    std::vector<FwdOp> ops;
    auto chainOps = [&](uint32_t ic) {
        ops.push_back({DIAG(ic + 1), OFF(ic), OFF(ic), (int32_t)ic});
        ops.push_back({RHS(ic + 1), OFF(ic), RHS(ic), (int32_t)ic});
    };
    {
        uint32_t ic = 0;
        for (const Junction& J : junction) {
            while (ic < J.index) chainOps(ic++);
            const std::vector<uint32_t>& grp = coupled[groupOf[J.index]];
            int64_t b = operandBase[J.index];
            int32_t p = (int32_t)J.index;
            if (J.rank == 1) {
                uint32_t far = grp.back();
                ops.push_back({DIAG(far), HJE(b + 1), HJE(b), p});
                ops.push_back({RHS(far), HJE(b + 1), RHS(J.index), p});
            } else if (J.rank == 2) {
                uint32_t f1 = grp[grp.size() - 2], f2 = grp[grp.size() - 1];
                ops.push_back({DIAG(f1), HJE(b + 1), HJE(b), p});
                ops.push_back({HJE(b + 4), HJE(b + 1), HJE(b + 2), p});
                ops.push_back({RHS(f1), HJE(b + 1), RHS(J.index), p});
                ops.push_back({HJE(b + 5), HJE(b + 3), HJE(b), p});
                ops.push_back({DIAG(f2), HJE(b + 3), HJE(b + 2), p});
                ops.push_back({RHS(f2), HJE(b + 3), RHS(J.index), p});
            } else {
                uint32_t rank = J.rank;
                size_t start = grp.size() - rank;
                for (uint32_t j = 0; j < rank; ++j) {
                    uint32_t far = grp[start + j];
                    ops.push_back({DIAG(far), HJE(b + 2 * j + 1), HJE(b + 2 * j), p});
                    ops.push_back({RHS(far), HJE(b + 2 * j + 1), RHS(J.index), p});
                }
                int64_t left = b + 1, target = b + 2 * rank, above;
                for (uint32_t i = 1; i < rank; ++i) {
                    above = b + 2 * i;
                    for (uint32_t j = 0; j < rank - i; ++j) {
                        ops.push_back({HJE(target), HJE(left), HJE(above), p});
                        above += 2;
                        target += 2;
                    }
                    left += 2;
                }
                target = b + 2 * rank + 1;
                above = b;
                for (uint32_t i = 1; i < rank; ++i) {
                    left = b + 2 * i + 1;
                    for (uint32_t j = 0; j < rank - i; ++j) {
                        ops.push_back({HJE(target), HJE(left), HJE(above), p});
                        target += 2;
                        left += 2;
                    }
                    above += 2;
                }
            }
            ++ic;
        }
        while (ic + 1 < N) chainOps(ic++);
    }
    // Pull form: ops grouped by owning row (order kept), rows by level.
    std::vector<uint32_t> flevel(N, 0);
    std::vector<std::vector<uint32_t>> rowOps(N);
    for (size_t k = 0; k < ops.size(); ++k) {
        uint32_t r = owner(ops[k].t);
        flevel[r] = std::max(flevel[r], flevel[ops[k].p] + 1);
        rowOps[r].push_back((uint32_t)k);
    }
    // Back substitution terms (HSolvePassive::backwardSubstitute).
    std::vector<std::vector<BwdTerm>> rowTerms(N);
    {
        std::vector<int64_t> junctionRank(N, 0);
        for (const Junction& J : junction) junctionRank[J.index] = J.rank;
        for (uint32_t i = 0; i < N; ++i) {
            uint32_t rank = (uint32_t)junctionRank[i];
            if (rank == 0) {
                if (i + 1 < N) rowTerms[i].push_back({OFF(i), (int32_t)(i + 1)});
                continue;
            }
            const std::vector<uint32_t>& grp = coupled[groupOf[i]];
            int64_t b = operandBase[i];
            if (rank == 1) {
                rowTerms[i].push_back({HJE(b), (int32_t)grp.back()});
            } else if (rank == 2) {
                rowTerms[i].push_back({HJE(b + 2), (int32_t)grp[grp.size() - 1]});
                rowTerms[i].push_back({HJE(b), (int32_t)grp[grp.size() - 2]});
            } else {
                size_t start = grp.size() - rank;
                for (uint32_t k = rank; k-- > 0;)
                    rowTerms[i].push_back({HJE(b + 2 * k), (int32_t)grp[start + k]});
            }
        }
    }
    std::vector<uint32_t> blevel(N, 0);
    for (uint32_t i = N; i-- > 0;)
        for (const BwdTerm& t : rowTerms[i]) blevel[i] = std::max(blevel[i], blevel[t.src] + 1);
    auto bucket = [&](const std::vector<uint32_t>& level, std::vector<uint32_t>& ptr,
                      std::vector<uint32_t>& rows, uint32_t& maxw) {
        uint32_t L = 0;
        for (uint32_t v : level) L = std::max(L, v + 1);
        ptr.assign(L + 1, 0);
        for (uint32_t v : level) ptr[v + 1]++;
        for (uint32_t l = 0; l < L; ++l) ptr[l + 1] += ptr[l];
        rows.resize(N);
        std::vector<uint32_t> fill(ptr.begin(), ptr.end() - 1);
        for (uint32_t i = 0; i < N; ++i) rows[fill[level[i]]++] = i;
        maxw = 0;
        for (uint32_t l = 0; l < L; ++l) maxw = std::max(maxw, ptr[l + 1] - ptr[l]);
    };
    bucket(flevel, P.fLevelPtr, P.fRows, P.maxLevelWidthF);
    bucket(blevel, P.bLevelPtr, P.bRows, P.maxLevelWidthB);
    P.fOpPtr.assign(N + 1, 0);
    for (uint32_t k = 0; k < N; ++k) {
        uint32_t r = P.fRows[k];
        P.fOpPtr[k + 1] = P.fOpPtr[k] + (uint32_t)rowOps[r].size();
        for (uint32_t o : rowOps[r]) P.fOps.push_back(ops[o]);
    }
    P.bTermPtr.assign(N + 1, 0);
    for (uint32_t k = 0; k < N; ++k) {
        uint32_t r = P.bRows[k];
        P.bTermPtr[k + 1] = P.bTermPtr[k] + (uint32_t)rowTerms[r].size();
        for (const BwdTerm& t : rowTerms[r]) P.bTerms.push_back(t);
    }
    // Cable runs of the two sweeps (a cable row eliminated by its
    // predecessor: the two chainOps updates and nothing else; substituted
    // from its successor: the one OFF term).
    {
        const int32_t offBase = (int32_t)(2 * N + H);
        const uint32_t LF = (uint32_t)P.fLevelPtr.size() - 1, LB = (uint32_t)P.bLevelPtr.size() - 1;
        auto fCable = [&](uint32_t l, uint32_t& row) {
            if (P.fLevelPtr[l + 1] - P.fLevelPtr[l] != 1) return false;
            const uint32_t k = P.fLevelPtr[l];
            row = P.fRows[k];
            if (row == 0 || P.fOpPtr[k + 1] - P.fOpPtr[k] != 2) return false;
            const FwdOp& a = P.fOps[P.fOpPtr[k]];
            const FwdOp& b = P.fOps[P.fOpPtr[k] + 1];
            const int32_t p = (int32_t)row - 1, off = offBase + p;
            return a.t == (int32_t)row && a.l == off && a.a == off && a.p == p &&
                   b.t == (int32_t)(N + row) && b.l == off && b.a == (int32_t)N + p && b.p == p;
        };
        auto bCable = [&](uint32_t l, uint32_t& row) {
            if (P.bLevelPtr[l + 1] - P.bLevelPtr[l] != 1) return false;
            const uint32_t k = P.bLevelPtr[l];
            row = P.bRows[k];
            if (row + 1 >= N || P.bTermPtr[k + 1] - P.bTermPtr[k] != 1) return false;
            const BwdTerm& t = P.bTerms[P.bTermPtr[k]];
            return t.coef == offBase + (int32_t)row && t.src == (int32_t)row + 1;
        };
        P.fRun.assign(LF, 0);
        P.fRunRow.assign(LF, 0);
        for (uint32_t l = 0, r0 = 0, r = 0; l < LF;) {
            if (!fCable(l, r0)) { ++l; continue; }
            uint32_t len = 1;
            while (l + len < LF && fCable(l + len, r) && r == r0 + len) ++len;
            P.fRun[l] = len;
            P.fRunRow[l] = r0;
            l += len;
        }
        P.bRun.assign(LB, 0);
        P.bRunRow.assign(LB, 0);
        for (uint32_t l = 0, i0 = 0, i = 0; l < LB;) {
            if (!bCable(l, i0)) { ++l; continue; }
            uint32_t len = 1;
            while (l + len < LB && bCable(l + len, i) && i + len == i0) ++len;
            P.bRun[l] = len;
            P.bRunRow[l] = i0;
            l += len;
        }
        // Waves of the forward sweep.  A level costs the group stepping the
        // cell one update chain of its longest row (a quotient and two FP64
        // operations per update, on a pipe that issues an FP64 warp
        // instruction every 64 cycles per SM sub-partition); a wave costs
        // one fused update.  Waves are kept where they are fewer than the
        // level programs' chained updates (runs of cable rows count one
        // update per row: their pivot stays in registers).
        std::vector<FwdPair> fused;
        std::vector<uint32_t> longestOf(LF, 0);
        for (uint32_t l = 0; l < LF; ++l) {
            uint32_t longest = 0;
            for (uint32_t k = P.fLevelPtr[l]; k < P.fLevelPtr[l + 1]; ++k) {
                uint32_t chain = 0;
                for (uint32_t o = P.fOpPtr[k]; o < P.fOpPtr[k + 1]; ++o) {
                    const FwdOp& a = P.fOps[o];
                    FwdPair f{a.t, a.a, -1, -1, a.l, a.p, 0, 0};
                    if (o + 1 < P.fOpPtr[k + 1] && a.t != a.l && a.t != a.p) {
                        const FwdOp& b = P.fOps[o + 1];
                        if (b.l == a.l && b.p == a.p) {
                            f.t2 = b.t;
                            f.a2 = b.a;
                            ++o;
                        }
                    }
                    fused.push_back(f);
                    ++chain;
                }
                longest = std::max(longest, chain);
            }
            longestOf[l] = longest;
        }
        double levelCost = 0;
        for (uint32_t l = 0; l < LF; ++l) {
            if (P.fRun[l]) {
                levelCost += P.fRun[l];
                l += P.fRun[l] - 1;
            } else {
                levelCost += longestOf[l];
            }
        }
        const size_t nEnt = 3 * (size_t)N + H;
        std::vector<int64_t> lastW(nEnt, -1), lastR(nEnt, -1);
        std::vector<uint32_t> wave(fused.size());
        uint32_t nWaves = 0;
        for (size_t k = 0; k < fused.size(); ++k) {
            const FwdPair& f = fused[k];
            const int32_t rd[6] = {f.l, f.p, f.a1, f.t1, f.a2, f.t2};
            int64_t w = 0;
            for (int32_t e : rd)
                if (e >= 0) w = std::max(w, lastW[e] + 1);
            for (int32_t e : {f.t1, f.t2})
                if (e >= 0) w = std::max(w, lastR[e] + 1);
            wave[k] = (uint32_t)w;
            for (int32_t e : rd)
                if (e >= 0) lastR[e] = std::max(lastR[e], w);
            for (int32_t e : {f.t1, f.t2})
                if (e >= 0) lastW[e] = w;
            nWaves = std::max(nWaves, (uint32_t)w + 1);
        }
        if (nWaves < levelCost) {
            P.fWavePtr.assign(nWaves + 1, 0);
            for (uint32_t w : wave) P.fWavePtr[w + 1]++;
            for (uint32_t w = 0; w < nWaves; ++w) P.fWavePtr[w + 1] += P.fWavePtr[w];
            P.fWaveOps.resize(fused.size());
            std::vector<uint32_t> fill(P.fWavePtr.begin(), P.fWavePtr.end() - 1);
            for (size_t k = 0; k < fused.size(); ++k) P.fWaveOps[fill[wave[k]]++] = fused[k];
        }
    }

    // readHHChannels (hsolve/HSolveActiveSetup.cpp:162-235)
    std::vector<std::vector<uint32_t>> chansOf(d.n_compt);
    for (uint32_t k = 0; k < d.n_chan; ++k) {
        if (d.chan_compt[k] >= d.n_compt) return fail("channel compartment out of range");
        chansOf[d.chan_compt[k]].push_back(k);
    }
    P.chanPtr.assign(N + 1, 0);
    P.chanSolverOf.assign(d.n_chan, -1);
    std::vector<uint32_t> chanCompt;
    for (uint32_t ic = 0; ic < N; ++ic) {
        for (uint32_t k : chansOf[P.modelOf[ic]]) {
            uint32_t q = (uint32_t)P.Gbar.size();
            P.chanSolverOf[k] = q;
            P.chanModel.push_back(k);
            chanCompt.push_back(ic);
            P.Gbar.push_back(d.chan_Gbar[k]);
            P.Ek.push_back(d.chan_Ek[k]);
            P.Xpow.push_back(d.chan_Xpower[k]);
            P.Ypow.push_back(d.chan_Ypower[k]);
            P.Zpow.push_back(d.chan_Zpower[k]);
            P.instant.push_back(d.chan_instant[k]);
            P.modulation.push_back(d.chan_modulation[k]);
            P.stateOff.push_back((int32_t)P.state0.size());
            if (d.chan_Xpower[k] > 0.0) P.state0.push_back(d.chan_X[k]);
            if (d.chan_Ypower[k] > 0.0) P.state0.push_back(d.chan_Y[k]);
            if (d.chan_Zpower[k] > 0.0) P.state0.push_back(d.chan_Z[k]);
        }
        P.chanPtr[ic + 1] = (uint32_t)P.Gbar.size();
    }
    const uint32_t C = (uint32_t)P.Gbar.size();
    P.C = C;
    P.G = (uint32_t)P.state0.size();

    // readGates (hsolve/HSolveActiveSetup.cpp:237-250)
    std::vector<int64_t> gateId;
    std::vector<int> gCaDepend;
    std::vector<int32_t> firstGate(C);
    for (uint32_t q = 0; q < C; ++q) {
        uint32_t k = P.chanModel[q];
        firstGate[q] = (int32_t)gateId.size();
        int32_t gx[3] = {d.chan_xgate[k], d.chan_ygate[k], d.chan_zgate[k]};
        double pw[3] = {d.chan_Xpower[k], d.chan_Ypower[k], d.chan_Zpower[k]};
        size_t first = gateId.size();
        for (int w = 0; w < 3; ++w)
            if (pw[w] > 0.0) {
                if (gx[w] < 0 || gx[w] >= (int32_t)d.n_gate) return fail("channel gate index out of range");
                gateId.push_back(gx[w]);
                gCaDepend.push_back(0);
            }
        if (d.chan_use_conc[k] && gateId.size() > first) gCaDepend.back() = 1;
    }

    // readCalcium (hsolve/HSolveActiveSetup.cpp:252-337)
    P.poolPtr.assign(N + 1, 0);
    P.poolSolverOf.assign(d.n_pool, -1);
    std::vector<int64_t> caConcIndex(d.n_pool, -1);
    std::vector<int64_t> caTargetIndex, caDependIndex;
    std::vector<uint32_t> caCount(N, 0);
    {
        uint32_t ichan = 0;
        for (uint32_t ic = 0; ic < N; ++ic) {
            uint32_t nCa = (uint32_t)P.CaBasal.size();
            for (; ichan < P.chanPtr[ic + 1]; ++ichan) {
                uint32_t k = P.chanModel[ichan];
                std::vector<int64_t> ids;
                bool nTarget = d.chan_ca_target[k] >= 0, nDepend = d.chan_ca_depend[k] >= 0;
                if (nTarget) ids.push_back(d.chan_ca_target[k]);
                else caTargetIndex.push_back(-1);
                if (nDepend) ids.push_back(d.chan_ca_depend[k]);
                else caDependIndex.push_back(-1);
                for (int64_t p : ids) {
                    if (p >= (int64_t)d.n_pool) return fail("channel pool index out of range");
                    if (caConcIndex[p] < 0) {
                        if (!(d.pool_tau[p] != 0.0)) return fail("CaConc tau must be non-zero");
                        caConcIndex[p] = caCount[ic]++;
                        P.poolSolverOf[p] = (int64_t)P.CaBasal.size();
                        P.poolModel.push_back((uint32_t)p);
                        P.CaBasal.push_back(d.pool_CaBasal[p]);
                        P.c0.push_back(d.pool_Ca[p] - d.pool_CaBasal[p]);
                        double tau = d.pool_tau[p], B = d.pool_B[p];
                        P.f1.push_back(4.0 / (2.0 + dt / tau) - 1.0);
                        P.f2.push_back(2.0 * B * dt / (2.0 + dt / tau));
                        P.ceiling.push_back(d.pool_ceiling[p]);
                        P.floor_.push_back(d.pool_floor[p]);
                    }
                }
                if (nTarget) caTargetIndex.push_back(caConcIndex[ids.front()] + nCa);
                if (nDepend) caDependIndex.push_back(caConcIndex[ids.back()]);
            }
            P.poolPtr[ic + 1] = (uint32_t)P.CaBasal.size();
        }
    }
    const uint32_t Pn = (uint32_t)P.CaBasal.size();
    P.P = Pn;
    P.caTarget.resize(C);
    for (uint32_t q = 0; q < C; ++q) {
        int64_t t = caTargetIndex[q];
        if (t >= (int64_t)Pn) return fail("channel feeds a calcium pool outside the solver");
        P.caTarget[q] = (int32_t)t;
    }
    P.feedPtr.assign(Pn + 1, 0);
    for (uint32_t q = 0; q < C; ++q) if (P.caTarget[q] >= 0) P.feedPtr[P.caTarget[q] + 1]++;
    for (uint32_t p = 0; p < Pn; ++p) P.feedPtr[p + 1] += P.feedPtr[p];
    P.feedChan.resize(P.feedPtr[Pn]);
    {
        std::vector<uint32_t> fill(P.feedPtr.begin(), P.feedPtr.end() - 1);
        for (uint32_t q = 0; q < C; ++q) if (P.caTarget[q] >= 0) P.feedChan[fill[P.caTarget[q]]++] = q;
    }

    // createLookupTables (hsolve/HSolveActiveSetup.cpp:339-526)
    {
        std::set<int64_t> caSet, vSet;
        for (size_t g = 0; g < gateId.size(); ++g) (gCaDepend[g] ? caSet : vSet).insert(gateId[g]);
        std::vector<int64_t> caGate(caSet.begin(), caSet.end()), vGate(vSet.begin(), vSet.end());
        std::map<int64_t, uint32_t> species;
        for (size_t i = 0; i < caGate.size(); ++i) species[caGate[i]] = (uint32_t)i;
        for (size_t i = 0; i < vGate.size(); ++i) species[vGate[i]] = (uint32_t)i;
        P.vMin = DBL_MAX; P.vMax = DBL_MIN; double vDx = DBL_MAX;
        P.caMin = DBL_MAX; P.caMax = DBL_MIN; double caDx = DBL_MAX;
        for (int64_t g : caGate) {
            const HsGateTable& t = d.gate[g];
            double dx = (t.max - t.min) / t.divs;
            if (t.min < P.caMin) P.caMin = t.min;
            if (t.max > P.caMax) P.caMax = t.max;
            if (dx < caDx) caDx = dx;
        }
        P.caDiv = (int)((P.caMax - P.caMin) / caDx + 0.5);
        for (int64_t g : vGate) {
            const HsGateTable& t = d.gate[g];
            double dx = (t.max - t.min) / t.divs;
            if (t.min < P.vMin) P.vMin = t.min;
            if (t.max > P.vMax) P.vMax = t.max;
            if (dx < vDx) vDx = dx;
        }
        P.vDiv = (int)((P.vMax - P.vMin) / vDx + 0.5);
        if (!vGate.empty() && P.vDiv < 1) return fail("voltage table has no divisions");
        if (!caGate.empty() && P.caDiv < 1) return fail("calcium table has no divisions");
        initTable(P.caTable, P.caMin, P.caMax, caGate.empty() ? 0 : (uint32_t)P.caDiv, (uint32_t)caGate.size());
        initTable(P.vTable, P.vMin, P.vMax, vGate.empty() ? 0 : (uint32_t)P.vDiv, (uint32_t)vGate.size());
        for (int pass = 0; pass < 2; ++pass) {
            Table& t = pass ? P.vTable : P.caTable;
            const std::vector<int64_t>& set = pass ? vGate : caGate;
            if (set.empty()) continue;
            double gmin = pass ? P.vMin : P.caMin, gmax = pass ? P.vMax : P.caMax;
            unsigned gdivs = (unsigned)(pass ? P.vDiv : P.caDiv);
            double gdx = (gmax - gmin) / gdivs;
            std::vector<double> A(gdivs + 1), B(gdivs + 1);
            for (size_t s = 0; s < set.size(); ++s) {
                const HsGateTable& g = d.gate[set[s]];
                if (g.min == gmin && g.max == gmax && g.divs == gdivs) {
                    addColumns(t, (uint32_t)s, g.A, g.B, (size_t)g.divs + 1);
                } else {
                    for (size_t i = 0; i <= gdivs; ++i) gateLookupBoth(g, gmin + gdx * i, &A[i], &B[i]);
                    addColumns(t, (uint32_t)s, A.data(), B.data(), A.size());
                }
            }
        }
        std::vector<int32_t> column(gateId.size());
        for (size_t g = 0; g < gateId.size(); ++g) column[g] = 2 * (int32_t)species[gateId[g]];
        P.colX.assign(C, -1); P.colY.assign(C, -1); P.colZ.assign(C, -1); P.zSrc.assign(C, -1);
        for (uint32_t q = 0; q < C; ++q) {
            int32_t g = firstGate[q];
            if (P.Xpow[q] > 0.0) P.colX[q] = column[g++];
            if (P.Ypow[q] > 0.0) P.colY[q] = column[g++];
            if (P.Zpow[q] > 0.0) {
                P.colZ[q] = column[g++];
                int64_t cd = caDependIndex[q];
                uint32_t ic = chanCompt[q];
                if (cd >= 0) {
                    // caRowCompt_[cd] holds the row of this compartment's cd-th pool
                    if (cd >= (int64_t)(P.poolPtr[ic + 1] - P.poolPtr[ic]))
                        return fail("Ca-dependent gate reads a pool outside its compartment");
                    P.zSrc[q] = (int32_t)(P.poolPtr[ic] + cd);
                }
            }
        }
    }

    // external tick-4 objects
    P.K2 = d.n_chan2d;
    for (uint32_t g = 0; g < d.n_gate2d; ++g) {
        const HsGate2DTable& t = d.gate2d[g];
        Gate2D G2;
        G2.xmin = t.xmin; G2.xmax = t.xmax; G2.ymin = t.ymin; G2.ymax = t.ymax;
        G2.nx = t.xdivs + 1; G2.ny = t.ydivs + 1;
        G2.invDx = (double)t.xdivs / (t.xmax - t.xmin);
        G2.invDy = (double)t.ydivs / (t.ymax - t.ymin);
        G2.srcA = t.A;
        G2.srcB = t.B;
        if (opt.copyTables2d) {
            G2.AB.resize((size_t)G2.nx * G2.ny * 2);
            for (size_t i = 0; i < (size_t)G2.nx * G2.ny; ++i) {
                G2.AB[2 * i] = t.A[i];
                G2.AB[2 * i + 1] = t.B[i];
            }
        }
        P.gates2d.push_back(std::move(G2));
    }
    for (uint32_t k = 0; k < d.n_chan2d; ++k) {
        if (d.c2d_compt[k] >= d.n_compt || P.hinesOf[d.c2d_compt[k]] < 0)
            return fail("HHChannel2D compartment not in the tree");
        if (d.c2d_xgate[k] < 0 || d.c2d_xgate[k] >= (int32_t)d.n_gate2d)
            return fail("HHChannel2D gate index out of range");
        int d0, d1;
        switch (d.c2d_xindex[k]) {
            case HS_DEP_VOLT: d0 = 0; d1 = -1; break;
            case HS_DEP_C1: d0 = 1; d1 = -1; break;
            case HS_DEP_C2: d0 = 2; d1 = -1; break;
            case HS_DEP_VOLT_C1: d0 = 0; d1 = 1; break;
            case HS_DEP_VOLT_C2: d0 = 0; d1 = 2; break;
            case HS_DEP_C1_C2: d0 = 1; d1 = 2; break;
            default: return fail("HHChannel2D index code out of range");
        }
        int32_t c1 = -1, c2 = -1;
        if (d.c2d_conc1_pool[k] >= 0) {
            if (d.c2d_conc1_pool[k] >= (int32_t)d.n_pool || P.poolSolverOf[d.c2d_conc1_pool[k]] < 0)
                return fail("HHChannel2D conc1 pool is not taken by the solver");
            c1 = (int32_t)P.poolSolverOf[d.c2d_conc1_pool[k]];
        }
        if (d.c2d_conc2_pool[k] >= 0) {
            if (d.c2d_conc2_pool[k] >= (int32_t)d.n_pool || P.poolSolverOf[d.c2d_conc2_pool[k]] < 0)
                return fail("HHChannel2D conc2 pool is not taken by the solver");
            c2 = (int32_t)P.poolSolverOf[d.c2d_conc2_pool[k]];
        }
        P.c2dCompt.push_back((uint32_t)P.hinesOf[d.c2d_compt[k]]);
        P.c2dGbar.push_back(d.c2d_Gbar[k]);
        P.c2dEk.push_back(d.c2d_Ek[k]);
        P.c2dXpow.push_back(d.c2d_Xpower[k]);
        P.c2dMod.push_back(d.c2d_modulation[k]);
        P.c2dX0.push_back(d.c2d_X[k]);
        P.c2dGate.push_back(d.c2d_xgate[k]);
        P.c2dDep0.push_back(d0);
        P.c2dDep1.push_back(d1);
        P.c2dConc1.push_back(c1);
        P.c2dConc2.push_back(c2);
        P.c2dInstant.push_back(d.c2d_instant[k]);
    }
    P.S = d.n_syn;
    for (uint32_t k = 0; k < d.n_syn; ++k) {
        if (d.syn_compt[k] >= d.n_compt || P.hinesOf[d.syn_compt[k]] < 0)
            return fail("SynChan compartment not in the tree");
        if (!(d.syn_tau1[k] > 0.0) || d.syn_tau2[k] < 0.0) return fail("SynChan taus must be positive");
        P.synCompt.push_back((uint32_t)P.hinesOf[d.syn_compt[k]]);
        P.synGbar.push_back(d.syn_Gbar[k]);
        P.synEk.push_back(d.syn_Ek[k]);
        P.synTau1.push_back(d.syn_tau1[k]);
        P.synTau2.push_back(d.syn_tau2[k]);
        P.synMod.push_back(d.syn_modulation[k]);
    }
    {
        std::vector<uint32_t> order(d.n_event);
        for (uint32_t e = 0; e < d.n_event; ++e) {
            if (d.ev_syn[e] >= d.n_syn) return fail("event SynChan index out of range");
            order[e] = e;
        }
        std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
            if (d.ev_syn[a] != d.ev_syn[b]) return d.ev_syn[a] < d.ev_syn[b];
            return d.ev_time[a] < d.ev_time[b];
        });
        P.evPtr.assign(d.n_syn + 1, 0);
        for (uint32_t e : order) {
            P.evPtr[d.ev_syn[e] + 1]++;
            P.evTime.push_back(d.ev_time[e]);
            P.evW.push_back(d.ev_weight[e]);
        }
        for (uint32_t k = 0; k < d.n_syn; ++k) P.evPtr[k + 1] += P.evPtr[k];
    }
    // tick-4 send order per compartment: HHChannel2D in creation order, then
    // SynChans in reverse creation order (the reference clock's proc4 order).
    {
        std::vector<std::vector<int32_t>> ext(N);
        for (uint32_t k = 0; k < P.K2; ++k) ext[P.c2dCompt[k]].push_back((int32_t)k);
        for (uint32_t k = P.S; k-- > 0;) ext[P.synCompt[k]].push_back(-(int32_t)k - 1);
        P.extPtr.assign(N + 1, 0);
        for (uint32_t i = 0; i < N; ++i) {
            P.extPtr[i + 1] = P.extPtr[i] + (uint32_t)ext[i].size();
            P.extList.insert(P.extList.end(), ext[i].begin(), ext[i].end());
        }
    }
    P.SG = d.n_spikegen;
    for (uint32_t k = 0; k < d.n_spikegen; ++k) {
        if (d.sg_compt[k] >= d.n_compt || P.hinesOf[d.sg_compt[k]] < 0)
            return fail("SpikeGen compartment not in the tree");
        P.sgCompt.push_back((uint32_t)P.hinesOf[d.sg_compt[k]]);
        P.sgThreshold.push_back(d.sg_threshold[k]);
        P.sgRefract.push_back(d.sg_refractT[k]);
        P.sgEdge.push_back(d.sg_edge[k]);
    }
    for (uint32_t k = 0; k < d.n_stim; ++k) {
        if (d.stim_compt[k] >= d.n_compt || P.hinesOf[d.stim_compt[k]] < 0)
            return fail("stimulus compartment not in the tree");
        if (k && d.stim_step[k] < d.stim_step[k - 1]) return fail("stimulus schedule not sorted by step");
        P.stimStep.push_back(d.stim_step[k]);
        P.stimCompt.push_back((uint32_t)P.hinesOf[d.stim_compt[k]]);
        P.stimValue.push_back(d.stim_value[k]);
    }
    // tick-1 external calcium objects and their messages
    if (d.n_dif || d.n_dmsg) {
        const uint32_t n = d.n_dif;
        if (n && (!d.dif_kind || !d.difpar)) return fail("tick-1 objects without kinds or parameters");
        if (d.n_dmsg && (!d.dmsg_kind || !d.dmsg_src || !d.dmsg_dst)) return fail("tick-1 messages without arrays");
        P.nDif = n;
        P.difKind.assign(d.dif_kind, d.dif_kind + n);
        P.difPar.assign(d.difpar, d.difpar + (size_t)n * HS_DIF_NPAR);
        for (int32_t k : P.difKind)
            if (k < HS_DIF_SHELL || k > HS_DIF_PUMP) return fail("unknown tick-1 object kind");
        std::vector<std::vector<uint32_t>> byObj((size_t)n * kDifMsgKinds), byChan(P.C);
        for (uint32_t m = 0; m < d.n_dmsg; ++m) {
            const int kind = d.dmsg_kind[m];
            const uint32_t s = d.dmsg_src[m], t = d.dmsg_dst[m];
            if (kind == HS_DMSG_IK) {
                if (s >= d.n_chan || P.chanSolverOf[s] < 0) return fail("IkOut from a channel the solver does not hold");
                if (t >= n || P.difKind[t] != HS_DIF_SHELL) return fail("IkOut to an object that is not a DifShell");
                byChan[(size_t)P.chanSolverOf[s]].push_back(t);
                continue;
            }
            if (kind < HS_DMSG_OUTER || kind > HS_DMSG_PUMP || s >= n) return fail("bad tick-1 message");
            const int sk = P.difKind[s];
            bool ok;
            uint32_t dst = t;
            switch (kind) {
            case HS_DMSG_OUTER:
            case HS_DMSG_INNER: ok = sk != HS_DIF_PUMP && t < n && P.difKind[t] != HS_DIF_PUMP; break;
            case HS_DMSG_CONC_CHAN:
                ok = sk == HS_DIF_SHELL && t < d.n_chan && P.chanSolverOf[t] >= 0;
                if (ok) dst = (uint32_t)P.chanSolverOf[t];
                break;
            case HS_DMSG_CONC_BUF: ok = sk == HS_DIF_SHELL && t < n && P.difKind[t] == HS_DIF_BUFFER; break;
            case HS_DMSG_REACTION: ok = sk == HS_DIF_BUFFER && t < n && P.difKind[t] == HS_DIF_SHELL; break;
            default: ok = sk == HS_DIF_PUMP && t < n && P.difKind[t] == HS_DIF_SHELL; break;
            }
            if (!ok) return fail("tick-1 message between objects of the wrong kinds");
            byObj[(size_t)s * kDifMsgKinds + kind].push_back(dst);
        }
        P.difOff.assign(1, 0);
        for (const auto& v : byObj) {
            P.difDst.insert(P.difDst.end(), v.begin(), v.end());
            P.difOff.push_back((uint32_t)P.difDst.size());
        }
        P.ikOff.assign(1, 0);
        for (const auto& v : byChan) {
            P.ikDst.insert(P.ikDst.end(), v.begin(), v.end());
            P.ikOff.push_back((uint32_t)P.ikDst.size());
        }
    }
    return true;
}

}  // namespace hsg
