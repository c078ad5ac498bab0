// moose_hsolve_bridge.cpp -- the MOOSE-side half of the drop-in boundary.
//
// Compiled inside a MOOSE source tree (it includes MOOSE's own headers), this
// file turns a MOOSE `HSolve` whose `HSolveActive::setup` has run
// (hsolve/HSolve.cpp:286-334 -> hsolve/HSolveActiveSetup.cpp:17-41) into the
// `HsCellDesc` that `hs_create` takes (include/moose_gb300.h).  It reads the
// solver's own vectors -- the tree walk and passive store
// (hsolve/HSolvePassive.cpp:45-205), the channels, gate Ids, Ca pools and
// their caTarget/caDepend links (hsolve/HSolveActiveSetup.cpp:162-337), the
// SynChans and SpikeGens (:538-577) -- and, through the Ids the solver keeps,
// the fields it does not store itself (gate tables, leakage channels, pool
// tau/B, the external HHChannel2D objects on each compartment's `channel`
// message).
//
// Model index = the solver's Hines index.  The description lists the
// compartments in the solver's order (compartmentId_), so the caller's
// Id -> index map is HSolve's own localIndex (hsolve/HSolveInterface.cpp:
// 23-36), channels in channel_ order, pools in caConc_ order.  Each
// compartment's parent is the node above it in the solver's tree_ (the
// depth-first tree the walk built, rooted at the walk's start leaf, Hines
// index N-1), children connected in increasing index: so the description's
// own walk from seed N-1 visits the compartments in exactly the solver's
// order and the Hines numbering is the identity.
//
// `fillCellDesc` is what a modified `HSolve::setup` calls after
// `HSolveActive::setup` and before `hs_create(&desc, seed, dt_, ...)`.  The
// solver's vectors are protected members of HSolveActive/HSolvePassive; a
// member function of HSolve reads them directly.  Kept outside the class
// here (no MOOSE header is edited), the reads go through pointers to
// members taken inside a class derived from HSolve, which the language
// allows for any HSolve object.
//
// Synaptic events are not part of the description: they arrive at run time
// through Synapse::addSpike -> SimpleSynHandler::addSpike, which the
// integration forwards to hs_push_events.  Basal-inject changes between
// `moose.start` calls reach the solver as zombie field writes
// (hs_set_field), so the description carries no stimulus schedule.

#include <algorithm>
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

// MOOSE headers, in the order the solver's own translation units use
#include "basecode/header.h"
#include "hsolve/HSolveStruct.h"
#include "hsolve/HinesMatrix.h"
#include "hsolve/HSolvePassive.h"
#include "hsolve/RateLookup.h"
#include "hsolve/HSolveActive.h"
#include "hsolve/HSolve.h"
#include "hsolve/HSolveUtils.h"
#include "biophysics/SymCompartment.h"
#include "shell/Neutral.h"

#include "moose_gb300.h"

namespace moose_gb300_bridge {

// Storage behind one HsCellDesc: every array the description points into.
struct HsCellDescStore {
    std::vector<int32_t> parent, link;
    std::vector<double> Ra, Rm, Cm, Em, initVm, Vm, inject;
    std::vector<uint32_t> leak_compt;
    std::vector<double> leak_Ek, leak_Gk;
    std::vector<std::vector<double>> gateA, gateB;
    std::vector<HsGateTable> gate;
    std::vector<uint32_t> chan_compt;
    std::vector<double> chan_Gbar, chan_Ek, chan_Xpower, chan_Ypower, chan_Zpower, chan_modulation;
    std::vector<int32_t> chan_xgate, chan_ygate, chan_zgate, chan_instant, chan_use_conc;
    std::vector<double> chan_X, chan_Y, chan_Z;
    std::vector<int32_t> chan_ca_target, chan_ca_depend;
    std::vector<uint32_t> pool_compt;
    std::vector<double> pool_Ca, pool_CaBasal, pool_tau, pool_B, pool_ceiling, pool_floor;
    std::vector<std::vector<double>> g2dA, g2dB;
    std::vector<HsGate2DTable> gate2d;
    std::vector<uint32_t> c2d_compt;
    std::vector<double> c2d_Gbar, c2d_Ek, c2d_Xpower, c2d_modulation, c2d_X;
    std::vector<int32_t> c2d_xgate, c2d_xindex, c2d_conc1_pool, c2d_conc2_pool, c2d_instant;
    std::vector<uint32_t> syn_compt;
    std::vector<double> syn_Gbar, syn_Ek, syn_tau1, syn_tau2, syn_modulation;
    std::vector<uint32_t> sg_compt;
    std::vector<double> sg_threshold, sg_refractT;
    std::vector<int32_t> sg_edge;
    std::vector<int32_t> dif_kind;
    std::vector<double> difpar;
    std::vector<int32_t> dmsg_kind;
    std::vector<uint32_t> dmsg_src, dmsg_dst;
    // the MOOSE objects behind each index, for the caller's Id -> index maps
    std::vector<Id> comptId, chanId, poolId, chan2dId, synId, spikeGenId, difId;
    uint32_t seed = 0;
    HsCellDesc desc{};
};

namespace {

// Reads of HSolve's protected vectors through pointers to members named in
// a derived class.
struct SolverView : public HSolve {
    static const vector<Id>& compartmentId(const HSolve& h) { return h.*(&SolverView::compartmentId_); }
    static const vector<TreeNodeStruct>& tree(const HSolve& h) { return h.*(&SolverView::tree_); }
    static const vector<double>& V(const HSolve& h) { return h.*(&SolverView::V_); }
    static const map<unsigned int, InjectStruct>& inject(const HSolve& h) { return h.*(&SolverView::inject_); }
    static const vector<ChannelStruct>& channel(const HSolve& h) { return h.*(&SolverView::channel_); }
    static const vector<CurrentStruct>& current(const HSolve& h) { return h.*(&SolverView::current_); }
    static const vector<double>& state(const HSolve& h) { return h.*(&SolverView::state_); }
    static const vector<unsigned int>& chan2compt(const HSolve& h) { return h.*(&SolverView::chan2compt_); }
    static const vector<unsigned int>& chan2state(const HSolve& h) { return h.*(&SolverView::chan2state_); }
    static const vector<Id>& channelId(const HSolve& h) { return h.*(&SolverView::channelId_); }
    static const vector<Id>& gateId(const HSolve& h) { return h.*(&SolverView::gateId_); }
    static const vector<LookupRow>& caRowCompt(const HSolve& h) { return h.*(&SolverView::caRowCompt_); }
    static const vector<LookupRow*>& caRow(const HSolve& h) { return h.*(&SolverView::caRow_); }
    static const vector<CaConcStruct>& caConc(const HSolve& h) { return h.*(&SolverView::caConc_); }
    static const vector<Id>& caConcId(const HSolve& h) { return h.*(&SolverView::caConcId_); }
    static const vector<double>& caActivation(const HSolve& h) { return h.*(&SolverView::caActivation_); }
    static const vector<double*>& caTarget(const HSolve& h) { return h.*(&SolverView::caTarget_); }
    static const vector<unsigned int>& caCount(const HSolve& h) { return h.*(&SolverView::caCount_); }
    static const vector<SynChanStruct>& synchan(const HSolve& h) { return h.*(&SolverView::synchan_); }
    static const vector<SpikeGenStruct>& spikegen(const HSolve& h) { return h.*(&SolverView::spikegen_); }
};

template <class T>
const T* ptr(const std::vector<T>& v) {
    return v.empty() ? nullptr : v.data();
}

int xindexCode(const string& s) {
    static const char* names[] = {"VOLT_INDEX", "C1_INDEX", "C2_INDEX", "VOLT_C1_INDEX", "VOLT_C2_INDEX",
                                  "C1_C2_INDEX"};
    for (int i = 0; i < 6; ++i)
        if (s == names[i]) return i;
    return -1;
}

// useConcentration of the channel whose last gate is `gate`.  setup's
// readGates read it from the channel before the zombie took the channel's
// place (hsolve/HSolveActiveSetup.cpp:237-250) and cleanup() dropped it
// afterwards; the zombie does not keep it (biophysics/HHChannelBase.cpp
// zombify).  The solver's gate Ids are the prototype gates the channels were
// copied from (HSolveUtils::gates with getOriginals), and a prototype channel
// is not zombified, so it still holds the flag.  A channel that is its own
// prototype is zombified too: for it the flag is taken to be whether its Z
// gate reads a pool.
int useConcentration(const Id& gate, bool readsPool) {
    const ObjId owner = Neutral::parent(ObjId(gate));
    if (!owner.bad() && owner.element()->cinfo()->name() == "HHChannel")
        return Field<int>::get(owner, "useConcentration");
    return readsPool ? 1 : 0;
}

}  // namespace

// Fills `out` from `hs`, on which HSolveActive::setup has run.  Returns 0, or
// HS_EINVAL with `err` set when the solver holds something the description
// cannot express.
int fillCellDesc(const HSolve& hs, HsCellDescStore& out, std::string& err) {
    typedef SolverView S;
    out = HsCellDescStore();
    const vector<Id>& cid = S::compartmentId(hs);
    const vector<TreeNodeStruct>& tree = S::tree(hs);
    const uint32_t N = (uint32_t)cid.size();
    if (N == 0 || tree.size() != N) {
        err = "the solver has no compartments (setup has not run)";
        return HS_EINVAL;
    }
    // ---- compartments, in the solver's order
    out.comptId = cid;
    out.parent.assign(N, -1);
    for (uint32_t i = 0; i < N; ++i)
        for (unsigned int c : tree[i].children) out.parent[c] = (int32_t)i;
    // the message each compartment hangs on: HSolveUtils::children takes the
    // parent's axial, distalOut and cylinderOut targets (in that order), and
    // HSolveUtils::adjacent puts the parent between them by the link's kind.
    // The compartments are zombies by now (ZombieCompartment has no
    // distalOut/cylinderOut Finfo), but a zombie swap keeps the element's
    // messages, so they are read with SymCompartment's own Finfos; only
    // targets that are the node's children in tree_ count.
    out.link.assign(N, HS_LINK_AXIAL);
    {
        const Cinfo* sym = SymCompartment::initCinfo();
        const Finfo* byKind[] = {nullptr, sym->findFinfo("distalOut"), sym->findFinfo("cylinderOut")};
        for (uint32_t i = 0; i < N; ++i) {
            if (tree[i].children.empty()) continue;
            vector<Id> axial;
            HSolveUtils::targets(cid[i], "axial", axial);
            for (int k = HS_LINK_CYLINDER; k >= HS_LINK_DISTAL; --k) {
                vector<Id> t;
                if (byKind[k]) cid[i].element()->getNeighbors(t, byKind[k]);
                for (unsigned int c : tree[i].children)
                    if (std::find(t.begin(), t.end(), cid[c]) != t.end()) out.link[c] = k;
            }
            for (unsigned int c : tree[i].children)
                if (std::find(axial.begin(), axial.end(), cid[c]) != axial.end()) out.link[c] = HS_LINK_AXIAL;
        }
    }
    const vector<double>& V = S::V(hs);
    for (uint32_t i = 0; i < N; ++i) {
        out.Ra.push_back(tree[i].Ra);
        out.Rm.push_back(tree[i].Rm);
        out.Cm.push_back(tree[i].Cm);
        out.Em.push_back(tree[i].Em);
        out.initVm.push_back(tree[i].initVm);
        out.Vm.push_back(V[i]);
    }
    out.inject.assign(N, 0.0);
    for (const auto& kv : S::inject(hs)) out.inject[kv.first] = kv.second.injectBasal;
    out.seed = N - 1;      // the start leaf of the solver's walk
    // ---- leakage channels (HSolvePassive::initialize sums them per compartment)
    for (uint32_t i = 0; i < N; ++i) {
        vector<Id> leak;
        HSolveUtils::leakageChannels(cid[i], leak);
        for (const Id& l : leak) {
            out.leak_compt.push_back(i);
            out.leak_Ek.push_back(Field<double>::get(l, "Ek"));
            out.leak_Gk.push_back(Field<double>::get(l, "Gk"));
        }
    }
    // ---- HHChannels and their gates
    const vector<ChannelStruct>& ch = S::channel(hs);
    const vector<CurrentStruct>& cur = S::current(hs);
    const vector<double>& state = S::state(hs);
    const vector<Id>& gid = S::gateId(hs);
    std::map<Id, int32_t> gateIndex;
    size_t gcur = 0;
    auto gateOf = [&](double power) -> int32_t {
        if (!(power > 0.0)) return -1;
        if (gcur >= gid.size()) return -2;
        const Id g = gid[gcur++];
        auto it = gateIndex.find(g);
        if (it != gateIndex.end()) return it->second;
        const int32_t k = (int32_t)out.gateA.size();
        gateIndex[g] = k;
        out.gateA.push_back(Field<vector<double>>::get(g, "tableA"));
        out.gateB.push_back(Field<vector<double>>::get(g, "tableB"));
        const double mn = Field<double>::get(g, "min"), mx = Field<double>::get(g, "max");
        out.gate.push_back(HsGateTable{mn, mx, 0, nullptr, nullptr});
        return k;
    };
    out.chanId = S::channelId(hs);
    const vector<unsigned int>& c2c = S::chan2compt(hs);
    const vector<unsigned int>& c2s = S::chan2state(hs);
    // the first pool of each compartment (pools are created compartment by
    // compartment; caDependIndex_ counts from the compartment's first pool)
    const vector<unsigned int>& caCount = S::caCount(hs);
    std::vector<uint32_t> poolBase(N + 1, 0);
    for (uint32_t i = 0; i < N; ++i) poolBase[i + 1] = poolBase[i] + (i < caCount.size() ? caCount[i] : 0);
    const vector<double>& act = S::caActivation(hs);
    const vector<double*>& tgt = S::caTarget(hs);
    const vector<LookupRow*>& caRow = S::caRow(hs);
    const vector<LookupRow>& caRowCompt = S::caRowCompt(hs);
    size_t zrow = 0;
    for (size_t k = 0; k < ch.size(); ++k) {
        const ChannelStruct& c = ch[k];
        out.chan_compt.push_back(c2c[k]);
        out.chan_Gbar.push_back(c.Gbar_);
        out.chan_Ek.push_back(cur[k].Ek);
        out.chan_Xpower.push_back(c.Xpower_);
        out.chan_Ypower.push_back(c.Ypower_);
        out.chan_Zpower.push_back(c.Zpower_);
        out.chan_instant.push_back(c.instant_);
        out.chan_modulation.push_back(c.modulation_);
        const size_t g0 = gcur;
        out.chan_xgate.push_back(gateOf(c.Xpower_));
        out.chan_ygate.push_back(gateOf(c.Ypower_));
        out.chan_zgate.push_back(gateOf(c.Zpower_));
        // the pool the Z gate reads (caRow_: one entry per channel with a Z
        // gate, pointing at the compartment's row buffer of that pool)
        int32_t depPool = -1;
        if (c.Zpower_ > 0.0) {
            const LookupRow* r = zrow < caRow.size() ? caRow[zrow] : nullptr;
            ++zrow;
            if (r) depPool = (int32_t)(poolBase[c2c[k]] + (uint32_t)(r - caRowCompt.data()));
        }
        out.chan_ca_depend.push_back(depPool);
        out.chan_use_conc.push_back(gcur > g0 ? useConcentration(gid[gcur - 1], depPool >= 0) : 0);
        size_t s = c2s[k];
        out.chan_X.push_back(c.Xpower_ > 0.0 ? state[s++] : 0.0);
        out.chan_Y.push_back(c.Ypower_ > 0.0 ? state[s++] : 0.0);
        out.chan_Z.push_back(c.Zpower_ > 0.0 ? state[s++] : 0.0);
        out.chan_ca_target.push_back(tgt[k] ? (int32_t)(tgt[k] - act.data()) : -1);
    }
    if (gcur != gid.size() || std::find(out.chan_xgate.begin(), out.chan_xgate.end(), -2) != out.chan_xgate.end() ||
        std::find(out.chan_ygate.begin(), out.chan_ygate.end(), -2) != out.chan_ygate.end() ||
        std::find(out.chan_zgate.begin(), out.chan_zgate.end(), -2) != out.chan_zgate.end()) {
        err = "gate Ids do not match the channels' powers";
        return HS_EINVAL;
    }
    for (size_t g = 0; g < out.gate.size(); ++g) {
        if (out.gateA[g].size() < 2 || out.gateA[g].size() != out.gateB[g].size()) {
            err = "a gate table has fewer than 2 entries or A and B differ in length";
            return HS_EINVAL;
        }
        out.gate[g].divs = (uint32_t)out.gateA[g].size() - 1;
        out.gate[g].A = out.gateA[g].data();
        out.gate[g].B = out.gateB[g].data();
    }
    // ---- Ca pools, in caConc_ order
    const vector<CaConcStruct>& pools = S::caConc(hs);
    out.poolId = S::caConcId(hs);
    std::map<Id, int32_t> poolIndex;
    for (size_t p = 0; p < pools.size(); ++p) {
        uint32_t ic = 0;
        while (ic < N && poolBase[ic + 1] <= p) ++ic;
        out.pool_compt.push_back(ic);
        out.pool_Ca.push_back(pools[p].c_ + pools[p].CaBasal_);
        out.pool_CaBasal.push_back(pools[p].CaBasal_);
        out.pool_tau.push_back(Field<double>::get(out.poolId[p], "tau"));
        out.pool_B.push_back(Field<double>::get(out.poolId[p], "B"));
        out.pool_ceiling.push_back(pools[p].ceiling_);
        out.pool_floor.push_back(pools[p].floor_);
        poolIndex[out.poolId[p]] = (int32_t)p;
    }
    // the pool whose concOut feeds `msg` of an HHChannel2D (the pools are
    // zombified by now)
    const vector<string> poolClasses = {"CaConc", "ZombieCaConc"};
    auto poolOf = [&](const Id& chan, const char* msg) -> int32_t {
        vector<Id> src;
        HSolveUtils::targets(chan, msg, src, poolClasses);
        if (src.empty()) return -1;
        auto it = poolIndex.find(src.back());
        return it == poolIndex.end() ? -1 : it->second;
    };
    // ---- external HHChannel2D objects on each compartment's `channel` message
    std::map<Id, int32_t> gate2dIndex;
    for (uint32_t i = 0; i < N; ++i) {
        vector<Id> found, c2d;
        HSolveUtils::targets(cid[i], "channel", found, "HHChannel2D");
        // a channel that also takes the compartment's VmOut through its own
        // Vm message is reached twice through the shared `channel` Finfo
        for (const Id& c : found)
            if (std::find(c2d.begin(), c2d.end(), c) == c2d.end()) c2d.push_back(c);
        for (const Id& c : c2d) {
            const double xp = Field<double>::get(c, "Xpower");
            int32_t gi = -1;
            if (xp > 0.0) {
                const ObjId go(c.path() + "/gateX");     // the channel's X gate (HHGate2D)
                const Id gx = go.id;
                auto it = gate2dIndex.find(gx);
                if (it != gate2dIndex.end()) {
                    gi = it->second;
                } else {
                    const vector<vector<double>> A = Field<vector<vector<double>>>::get(go, "tableA");
                    const vector<vector<double>> B = Field<vector<vector<double>>>::get(go, "tableB");
                    if (A.empty() || A.size() != B.size() || A[0].size() < 1) {
                        err = "an HHChannel2D gate table is empty or A and B differ";
                        return HS_EINVAL;
                    }
                    std::vector<double> fa, fb;
                    for (size_t x = 0; x < A.size(); ++x) {
                        if (A[x].size() != A[0].size() || B[x].size() != A[0].size()) {
                            err = "an HHChannel2D gate table is ragged";
                            return HS_EINVAL;
                        }
                        fa.insert(fa.end(), A[x].begin(), A[x].end());
                        fb.insert(fb.end(), B[x].begin(), B[x].end());
                    }
                    gi = (int32_t)out.gate2d.size();
                    gate2dIndex[gx] = gi;
                    out.g2dA.push_back(std::move(fa));
                    out.g2dB.push_back(std::move(fb));
                    HsGate2DTable t{};
                    t.xmin = Field<double>::get(go, "xmin");
                    t.xmax = Field<double>::get(go, "xmax");
                    t.ymin = Field<double>::get(go, "ymin");
                    t.ymax = Field<double>::get(go, "ymax");
                    t.xdivs = (uint32_t)A.size() - 1;
                    t.ydivs = (uint32_t)A[0].size() - 1;
                    out.gate2d.push_back(t);
                }
            }
            const int32_t xi = xindexCode(Field<string>::get(c, "Xindex"));
            if (xp > 0.0 && xi < 0) {
                err = "unknown HHChannel2D Xindex";
                return HS_EINVAL;
            }
            out.chan2dId.push_back(c);
            out.c2d_compt.push_back(i);
            out.c2d_Gbar.push_back(Field<double>::get(c, "Gbar"));
            out.c2d_Ek.push_back(Field<double>::get(c, "Ek"));
            out.c2d_Xpower.push_back(xp);
            out.c2d_modulation.push_back(Field<double>::get(c, "modulation"));
            out.c2d_X.push_back(0.0);        // reinit sets X from the table at Vm = 0, conc = 0
            out.c2d_instant.push_back(0);    // HHChannel2D has no instant gates
            out.c2d_xgate.push_back(gi);
            out.c2d_xindex.push_back(xi < 0 ? 0 : xi);
            out.c2d_conc1_pool.push_back(poolOf(c, "concen"));
            out.c2d_conc2_pool.push_back(poolOf(c, "concen2"));
        }
    }
    for (size_t g = 0; g < out.gate2d.size(); ++g) {
        out.gate2d[g].A = out.g2dA[g].data();
        out.gate2d[g].B = out.g2dB[g].data();
    }
    // ---- SynChans (readSynapses) and SpikeGens
    for (const SynChanStruct& s : S::synchan(hs)) {
        out.synId.push_back(s.elm_);
        out.syn_compt.push_back(s.compt_);
        out.syn_Gbar.push_back(Field<double>::get(s.elm_, "Gbar"));
        out.syn_Ek.push_back(Field<double>::get(s.elm_, "Ek"));
        out.syn_tau1.push_back(Field<double>::get(s.elm_, "tau1"));
        out.syn_tau2.push_back(Field<double>::get(s.elm_, "tau2"));
        out.syn_modulation.push_back(Field<double>::get(s.elm_, "modulation"));
    }
    for (const SpikeGenStruct& g : S::spikegen(hs)) {
        const ObjId o = g.e_.objId();
        out.spikeGenId.push_back(o.id);
        out.sg_compt.push_back((uint32_t)(g.Vm_ - V.data()));
        out.sg_threshold.push_back(Field<double>::get(o, "threshold"));
        out.sg_refractT.push_back(Field<double>::get(o, "refractT"));
        out.sg_edge.push_back(Field<bool>::get(o, "edgeTriggered") ? 1 : 0);
    }
    // ---- external calcium on tick 1: the DifShells the channels' IkOut
    // reaches or whose concentrationOut reaches a channel's concen, and every
    // DifShell, DifBuffer and MMPump connected to those through their
    // diffusion, concentration, reaction and pump messages
    {
        auto cls = [](const Id& x) { return x.element()->cinfo()->name(); };
        std::vector<Id> seen;
        std::vector<Id> todo;
        auto visit = [&](const Id& x) {
            const string c = cls(x);
            if ((c == "DifShell" || c == "DifBuffer" || c == "MMPump") &&
                std::find(seen.begin(), seen.end(), x) == seen.end()) {
                seen.push_back(x);
                todo.push_back(x);
            }
        };
        for (const Id& ch : out.chanId) {
            vector<Id> t;
            HSolveUtils::targets(ch, "IkOut", t, "DifShell");
            HSolveUtils::targets(ch, "concen", t, "DifShell");
            for (const Id& x : t) visit(x);
        }
        const char* links[] = {"innerDifSourceOut", "outerDifSourceOut", "concentrationOut", "reactionOut",
                               "PumpOut", "fluxFromOut", "fluxFromIn", "reaction", "mmPump", "concentration"};
        while (!todo.empty()) {
            const Id x = todo.back();
            todo.pop_back();
            for (const char* f : links) {
                vector<Id> t;
                HSolveUtils::targets(x, f, t);
                for (const Id& y : t) visit(y);
            }
        }
        // tick-1 process order: the order the objects were created in
        std::sort(seen.begin(), seen.end(), [](const Id& a, const Id& b) { return a.value() < b.value(); });
        out.difId = seen;
        std::map<Id, uint32_t> difIndex;
        for (uint32_t k = 0; k < seen.size(); ++k) difIndex[seen[k]] = k;
        std::map<Id, uint32_t> chanIndex;
        for (uint32_t k = 0; k < out.chanId.size(); ++k) chanIndex[out.chanId[k]] = k;
        for (uint32_t k = 0; k < seen.size(); ++k) {
            const Id& x = seen[k];
            const string c = cls(x);
            double p[HS_DIF_NPAR] = {0};
            if (c == "DifShell") {
                out.dif_kind.push_back(HS_DIF_SHELL);
                const char* f[] = {"Ceq", "D", "valence", "leak"};
                for (int i = 0; i < 4; ++i) p[i] = Field<double>::get(x, f[i]);
                p[4] = Field<unsigned int>::get(x, "shapeMode");
                const char* g[] = {"length", "diameter", "thickness", "volume", "outerArea", "innerArea"};
                for (int i = 0; i < 6; ++i) p[5 + i] = Field<double>::get(x, g[i]);
            } else if (c == "DifBuffer") {
                out.dif_kind.push_back(HS_DIF_BUFFER);
                const char* f[] = {"bTot", "kf", "kb", "D"};
                for (int i = 0; i < 4; ++i) p[i] = Field<double>::get(x, f[i]);
                p[4] = Field<unsigned int>::get(x, "shapeMode");
                const char* g[] = {"length", "diameter", "thickness", "volume", "outerArea", "innerArea", "activation"};
                for (int i = 0; i < 7; ++i) p[5 + i] = Field<double>::get(x, g[i]);
            } else {
                out.dif_kind.push_back(HS_DIF_PUMP);
                p[0] = Field<double>::get(x, "Vmax");
                p[1] = Field<double>::get(x, "Kd");
            }
            out.difpar.insert(out.difpar.end(), p, p + HS_DIF_NPAR);
        }
        auto emit = [&](int kind, uint32_t src, uint32_t dst) {
            out.dmsg_kind.push_back(kind);
            out.dmsg_src.push_back(src);
            out.dmsg_dst.push_back(dst);
        };
        // each object's sends, in message order per source finfo
        for (uint32_t k = 0; k < seen.size(); ++k) {
            const Id& x = seen[k];
            const struct { const char* finfo; int kind; } srcs[] = {
                {"innerDifSourceOut", HS_DMSG_INNER}, {"outerDifSourceOut", HS_DMSG_OUTER},
                {"concentrationOut", HS_DMSG_CONC_CHAN}, {"reactionOut", HS_DMSG_REACTION},
                {"PumpOut", HS_DMSG_PUMP}};
            for (const auto& s : srcs) {
                vector<Id> t;
                HSolveUtils::targets(x, s.finfo, t);
                for (const Id& y : t) {
                    auto di = difIndex.find(y);
                    auto ci = chanIndex.find(y);
                    if (s.kind == HS_DMSG_CONC_CHAN) {
                        if (ci != chanIndex.end()) emit(HS_DMSG_CONC_CHAN, k, ci->second);
                        else if (di != difIndex.end() && cls(y) == "DifBuffer") emit(HS_DMSG_CONC_BUF, k, di->second);
                    } else if (di != difIndex.end()) {
                        emit(s.kind, k, di->second);
                    }
                }
            }
        }
        // the solver's IkOut sends, channel order
        for (uint32_t q = 0; q < out.chanId.size(); ++q) {
            vector<Id> t;
            HSolveUtils::targets(out.chanId[q], "IkOut", t, "DifShell");
            for (const Id& y : t) emit(HS_DMSG_IK, q, difIndex[y]);
        }
    }
    // ---- the description
    HsCellDesc& d = out.desc;
    d.n_compt = N;
    d.parent = ptr(out.parent);
    d.link = ptr(out.link);
    d.Ra = ptr(out.Ra);
    d.Rm = ptr(out.Rm);
    d.Cm = ptr(out.Cm);
    d.Em = ptr(out.Em);
    d.initVm = ptr(out.initVm);
    d.Vm = ptr(out.Vm);
    d.inject = ptr(out.inject);
    d.n_leak = (uint32_t)out.leak_compt.size();
    d.leak_compt = ptr(out.leak_compt);
    d.leak_Ek = ptr(out.leak_Ek);
    d.leak_Gk = ptr(out.leak_Gk);
    d.n_gate = (uint32_t)out.gate.size();
    d.gate = ptr(out.gate);
    d.n_chan = (uint32_t)out.chan_compt.size();
    d.chan_compt = ptr(out.chan_compt);
    d.chan_Gbar = ptr(out.chan_Gbar);
    d.chan_Ek = ptr(out.chan_Ek);
    d.chan_Xpower = ptr(out.chan_Xpower);
    d.chan_Ypower = ptr(out.chan_Ypower);
    d.chan_Zpower = ptr(out.chan_Zpower);
    d.chan_xgate = ptr(out.chan_xgate);
    d.chan_ygate = ptr(out.chan_ygate);
    d.chan_zgate = ptr(out.chan_zgate);
    d.chan_instant = ptr(out.chan_instant);
    d.chan_modulation = ptr(out.chan_modulation);
    d.chan_use_conc = ptr(out.chan_use_conc);
    d.chan_X = ptr(out.chan_X);
    d.chan_Y = ptr(out.chan_Y);
    d.chan_Z = ptr(out.chan_Z);
    d.chan_ca_target = ptr(out.chan_ca_target);
    d.chan_ca_depend = ptr(out.chan_ca_depend);
    d.n_pool = (uint32_t)out.pool_compt.size();
    d.pool_compt = ptr(out.pool_compt);
    d.pool_Ca = ptr(out.pool_Ca);
    d.pool_CaBasal = ptr(out.pool_CaBasal);
    d.pool_tau = ptr(out.pool_tau);
    d.pool_B = ptr(out.pool_B);
    d.pool_ceiling = ptr(out.pool_ceiling);
    d.pool_floor = ptr(out.pool_floor);
    d.n_gate2d = (uint32_t)out.gate2d.size();
    d.gate2d = ptr(out.gate2d);
    d.n_chan2d = (uint32_t)out.c2d_compt.size();
    d.c2d_compt = ptr(out.c2d_compt);
    d.c2d_Gbar = ptr(out.c2d_Gbar);
    d.c2d_Ek = ptr(out.c2d_Ek);
    d.c2d_Xpower = ptr(out.c2d_Xpower);
    d.c2d_xgate = ptr(out.c2d_xgate);
    d.c2d_xindex = ptr(out.c2d_xindex);
    d.c2d_conc1_pool = ptr(out.c2d_conc1_pool);
    d.c2d_conc2_pool = ptr(out.c2d_conc2_pool);
    d.c2d_instant = ptr(out.c2d_instant);
    d.c2d_modulation = ptr(out.c2d_modulation);
    d.c2d_X = ptr(out.c2d_X);
    d.n_syn = (uint32_t)out.syn_compt.size();
    d.syn_compt = ptr(out.syn_compt);
    d.syn_Gbar = ptr(out.syn_Gbar);
    d.syn_Ek = ptr(out.syn_Ek);
    d.syn_tau1 = ptr(out.syn_tau1);
    d.syn_tau2 = ptr(out.syn_tau2);
    d.syn_modulation = ptr(out.syn_modulation);
    d.n_event = 0;
    d.n_spikegen = (uint32_t)out.sg_compt.size();
    d.sg_compt = ptr(out.sg_compt);
    d.sg_threshold = ptr(out.sg_threshold);
    d.sg_refractT = ptr(out.sg_refractT);
    d.sg_edge = ptr(out.sg_edge);
    d.n_stim = 0;
    d.n_dif = (uint32_t)out.dif_kind.size();
    d.dif_kind = ptr(out.dif_kind);
    d.difpar = ptr(out.difpar);
    d.n_dmsg = (uint32_t)out.dmsg_kind.size();
    d.dmsg_kind = ptr(out.dmsg_kind);
    d.dmsg_src = ptr(out.dmsg_src);
    d.dmsg_dst = ptr(out.dmsg_dst);
    return 0;
}

}  // namespace moose_gb300_bridge

// ---------------------------------------------------------------------------
// C entry points for a caller that holds the HSolve only by path (a test
// driving the reference's own pymoose): the description of the HSolve at
// `hsolve_path` (null on failure, see hsb_last_error), valid until
// hsb_free_cell_desc; and the path of the MOOSE object behind an index of a
// description.

namespace {
std::map<const HsCellDesc*, std::unique_ptr<moose_gb300_bridge::HsCellDescStore>> g_stores;
std::string g_err;
}  // namespace

extern "C" __attribute__((visibility("default"))) const HsCellDesc* hsb_fill_cell_desc(const char* hsolve_path,
                                                                                      uint32_t* seed) {
    g_err.clear();
    ObjId o(hsolve_path ? std::string(hsolve_path) : std::string());
    if (o.bad() || o.element()->cinfo()->name() != "HSolve") {
        g_err = "no HSolve at that path";
        return nullptr;
    }
    const HSolve* hs = reinterpret_cast<const HSolve*>(o.data());
    std::unique_ptr<moose_gb300_bridge::HsCellDescStore> st(new moose_gb300_bridge::HsCellDescStore());
    if (moose_gb300_bridge::fillCellDesc(*hs, *st, g_err) != 0) return nullptr;
    if (seed) *seed = st->seed;
    const HsCellDesc* d = &st->desc;
    g_stores[d] = std::move(st);
    return d;
}

extern "C" __attribute__((visibility("default"))) void hsb_free_cell_desc(const HsCellDesc* d) {
    g_stores.erase(d);
}

extern "C" __attribute__((visibility("default"))) const char* hsb_last_error(void) { return g_err.c_str(); }

// kind: 0 compartment, 1 HHChannel, 2 pool, 3 HHChannel2D, 4 SynChan, 5 SpikeGen,
// 6 tick-1 external calcium object
extern "C" __attribute__((visibility("default"))) int hsb_object_path(const HsCellDesc* d, int kind,
                                                                      uint32_t index, char* buf, uint32_t cap) {
    auto it = g_stores.find(d);
    if (it == g_stores.end()) return -1;
    const moose_gb300_bridge::HsCellDescStore& st = *it->second;
    const std::vector<Id>* v[] = {&st.comptId, &st.chanId, &st.poolId, &st.chan2dId, &st.synId, &st.spikeGenId,
                                  &st.difId};
    if (kind < 0 || kind > 6 || index >= v[kind]->size() || !buf || cap == 0) return -1;
    const std::string p = (*v[kind])[index].path();
    const size_t n = std::min<size_t>(p.size(), cap - 1);
    p.copy(buf, n);
    buf[n] = '\0';
    return (int)p.size();
}
