// hs_batch_api.cpp -- batched HSolve: many cells in one persistent kernel.
//
// No counterpart in the reference (it runs one serial HSolve per cell).
// Cells are set up exactly as the drop-in sets one up (hs_plan.cpp), then:
//   FP64  : every cell keeps the drop-in's layout and exact arithmetic; one
//           warp steps one cell (bit-identical to the drop-in).
//   MIXED : the compact layout of hs_mixed.cuh (tree in BFS order with
//           junction nodes, FP32 channels, FP64 solve).
// Packing: cells are spread over one wave of CTAs (SMs x CTAs/SM) by
// longest-processing-time first on their compartment count, then over the
// warps of each CTA the same way.  The dt loop runs `steps_per_launch` steps
// per launch and, with use_graph, a whole process() call is one CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <new>
#include <queue>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "../../include/moose_gb300.h"
#include "hs_cell.h"
#include "hs_mixed.cuh"
#include "hs_plan.h"

namespace hsg {
int setLastError(int code, const std::string& msg);
cudaError_t uploadMixedTypes(const ChanType* ct, int nct, const C2dType* kt, int nkt, const SynType* st,
                             int nst, cudaStream_t s);
cudaError_t launchBatchStepMixed(const MixBatch& b, const uint32_t* warpCellPtr, const uint32_t* warpCells,
                                 uint32_t nWarps, uint32_t nsteps, uint32_t threadsPerCta, cudaStream_t st);
cudaError_t launchBatchReinitMixed(const MixBatch& b, const double* initVm, const float* c2dX0,
                                   const uint32_t* evStart, cudaStream_t st);
cudaError_t launchScatterInject(double* const* addr, uint8_t* const* flag, const double* val, uint32_t n,
                                cudaStream_t st);
}  // namespace hsg

using namespace hsg;

namespace {

int berr(int code, const std::string& m) { return setLastError(code, m); }
int cerr(cudaError_t e, const char* where) {
    return setLastError(HS_EDEVICE, std::string(where) + ": " + cudaGetErrorString(e));
}

uint64_t fnv(const void* p, size_t n, uint64_t h = 1469598103934665603ull) {
    const unsigned char* c = (const unsigned char*)p;
    for (size_t i = 0; i < n; ++i) h = (h ^ c[i]) * 1099511628211ull;
    return h;
}

struct DevBuf {
    std::vector<void*> ptrs;
    cudaError_t err = cudaSuccess;
    template <class T>
    T* alloc(size_t n) {
        void* p = nullptr;
        if (err == cudaSuccess) err = cudaMalloc(&p, (n ? n : 1) * sizeof(T));
        if (err == cudaSuccess) ptrs.push_back(p);
        return (T*)p;
    }
    template <class T>
    T* up(const std::vector<T>& v, cudaStream_t st) {
        T* p = alloc<T>(v.size());
        if (err == cudaSuccess && !v.empty())
            err = cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st);
        return p;
    }
    template <class T>
    T* zeros(size_t n, cudaStream_t st) {
        T* p = alloc<T>(n);
        if (err == cudaSuccess) err = cudaMemsetAsync(p, 0, (n ? n : 1) * sizeof(T), st);
        return p;
    }
    void freeAll() {
        for (void* p : ptrs) cudaFree(p);
        ptrs.clear();
    }
};

// Host mirror of the mixed layout needed after creation.
struct MixHost {
    std::vector<MixCellRange> cells;
    std::vector<std::vector<int64_t>> nodeOf;     // per cell: model compartment -> global node
    std::vector<std::vector<int64_t>> poolOf;     // per cell: model pool -> global pool
    std::vector<double> initVm;                   // per node
    std::vector<float> c2dX0;
    std::vector<uint32_t> evStart;                // per SynChan (global)
    std::vector<uint32_t> evEnd;
    std::vector<double> evTime, evW;              // per event (FP64 from the description)
    std::vector<double> synGbar, synTau1, synTau2, synEk, synMod;
    std::vector<SynType> synTypes;                // built at reinit
    std::vector<std::tuple<double, double, double>> synTypeKey;
    std::vector<uint8_t> synTypeOf;
    uint64_t nNodes = 0;
};

}  // namespace

struct HsBatch {
    int precision = HS_PREC_FP64;
    int device = 0;
    int nSm = 0;
    cudaStream_t st = nullptr;
    uint32_t nCells = 0;
    double dtSetup = 0, clockDt = 0;
    bool reinited = false;
    int caAdvance = 1;
    std::vector<CellPlan> plans;
    uint64_t nCompt = 0;
    // packing / tuning
    uint32_t threadsPerCta = 256, ctasPerSm = 4, stepsPerLaunch = 100;
    bool useGraph = true;
    uint32_t nWarps = 0, nCtas = 0;
    uint32_t *dWarpPtr = nullptr, *dWarpCells = nullptr;
    DevBuf buf;              // long-lived allocations
    DevBuf packBuf;          // packing arrays (replaced by retuning)
    // FP64
    Arena arena;
    std::vector<DevCell> dcs;
    DevCell* dDcs = nullptr;
    double* dInitVm = nullptr;
    double* dSynConst = nullptr;
    std::vector<size_t> initVmOff, synOff;
    // mixed
    MixBatch mb{};
    MixHost mh;
    double* dMixInitVm = nullptr;
    float* dMixC2dX0 = nullptr;
    uint32_t* dEvStart = nullptr;
    uint32_t* dEvStep = nullptr;
    float* dEvAct = nullptr;
    float* dSynNorm = nullptr;
    // recording
    std::vector<std::pair<uint32_t, uint32_t>> rec;
    DevBuf recBuf;
    double* recBase = nullptr;
    uint32_t recCap = 0, recStride = 1;
    // spikes
    uint32_t spikeCap = 1024;
    // inject targets
    DevBuf injBuf;
    double** dInjAddr = nullptr;
    uint8_t** dInjFlag = nullptr;
    double* dInjVal = nullptr;
    uint32_t nInjTargets = 0;
    std::vector<std::vector<int32_t>> injEntryOf;   // mixed: per cell, compartment -> entry
    // timing: event pairs around each stepping launch
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> evs;
    size_t evUsed = 0;
    double timedMs = 0;
    uint32_t timedLaunches = 0;
    // graph
    cudaGraphExec_t gexec = nullptr;
    uint32_t gSteps = 0;
    uint64_t stepsDone = 0;
};

namespace {

cudaError_t launchStep(HsBatch* b, uint32_t k) {
    if (b->precision == HS_PREC_FP64)
        return launchBatchStepFp64(b->dDcs, b->dWarpPtr, b->dWarpCells, b->nWarps, k, b->threadsPerCta, b->st);
    return launchBatchStepMixed(b->mb, b->dWarpPtr, b->dWarpCells, b->nWarps, k, b->threadsPerCta, b->st);
}

int repack(HsBatch* b) {
    b->packBuf.freeAll();
    b->packBuf.err = cudaSuccess;
    if (b->gexec) {
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
    }
    uint32_t warpsPerCta = b->threadsPerCta / 32;
    b->nCtas = std::max<uint32_t>(1, b->nSm * b->ctasPerSm);
    b->nWarps = b->nCtas * warpsPerCta;
    std::vector<double> cost(b->nCells);
    for (uint32_t c = 0; c < b->nCells; ++c) {
        const CellPlan& P = b->plans[c];
        cost[c] = P.N + 0.3 * P.C + 0.5 * P.S + 2.0 * (P.fLevelPtr.size() + P.bLevelPtr.size());
    }
    std::vector<uint32_t> order(b->nCells);
    for (uint32_t c = 0; c < b->nCells; ++c) order[c] = c;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) { return cost[x] > cost[y]; });
    using Item = std::pair<double, uint32_t>;
    std::priority_queue<Item, std::vector<Item>, std::greater<Item>> cta;
    for (uint32_t k = 0; k < b->nCtas; ++k) cta.push({0.0, k});
    std::vector<std::vector<uint32_t>> ctaCells(b->nCtas);
    for (uint32_t c : order) {
        Item it = cta.top();
        cta.pop();
        ctaCells[it.second].push_back(c);
        cta.push({it.first + cost[c], it.second});
    }
    std::vector<std::vector<uint32_t>> warpCells(b->nWarps);
    for (uint32_t k = 0; k < b->nCtas; ++k) {
        std::priority_queue<Item, std::vector<Item>, std::greater<Item>> wq;
        for (uint32_t w = 0; w < warpsPerCta; ++w) wq.push({0.0, k * warpsPerCta + w});
        for (uint32_t c : ctaCells[k]) {
            Item it = wq.top();
            wq.pop();
            warpCells[it.second].push_back(c);
            wq.push({it.first + cost[c], it.second});
        }
    }
    std::vector<uint32_t> ptr(b->nWarps + 1, 0), cells;
    for (uint32_t w = 0; w < b->nWarps; ++w) {
        ptr[w + 1] = ptr[w] + (uint32_t)warpCells[w].size();
        cells.insert(cells.end(), warpCells[w].begin(), warpCells[w].end());
    }
    b->dWarpPtr = b->packBuf.up(ptr, b->st);
    b->dWarpCells = b->packBuf.up(cells, b->st);
    if (b->packBuf.err == cudaSuccess) b->packBuf.err = cudaStreamSynchronize(b->st);
    if (b->packBuf.err != cudaSuccess) return cerr(b->packBuf.err, "batch packing");
    return HS_OK;
}

// ---- FP64 batch: drop-in layout per cell, shared tables ---------------------
int buildFp64(HsBatch* b, const HsCellDesc* cells) {
    const uint32_t nC = b->nCells;
    // shared V/Ca tables by content, 2-D tables by source identity
    std::map<std::pair<uint64_t, size_t>, const double*> tabDev;
    std::map<std::tuple<const double*, const double*, uint32_t, uint32_t>, uint64_t> g2dIndex;
    std::vector<double> g2dHost;
    std::vector<std::vector<uint64_t>> g2dOffs(nC);
    for (uint32_t c = 0; c < nC; ++c) {
        const CellPlan& P = b->plans[c];
        for (uint32_t g = 0; g < P.gates2d.size(); ++g) {
            const Gate2D& G = P.gates2d[g];
            auto key = std::make_tuple(G.srcA, G.srcB, G.nx, G.ny);
            auto it = g2dIndex.find(key);
            if (it == g2dIndex.end()) {
                uint64_t off = g2dHost.size();
                size_t n = (size_t)G.nx * G.ny;
                g2dHost.resize(off + 2 * n);
                for (size_t i = 0; i < n; ++i) {
                    g2dHost[off + 2 * i] = G.srcA[i];
                    g2dHost[off + 2 * i + 1] = G.srcB[i];
                }
                it = g2dIndex.emplace(key, off).first;
            }
            g2dOffs[c].push_back(it->second);
        }
    }
    const double* g2dBase = b->buf.up(g2dHost, b->st);
    std::vector<const double*> vtab(nC), catab(nC);
    for (uint32_t c = 0; c < nC; ++c) {
        for (int pass = 0; pass < 2; ++pass) {
            const Table& T = pass ? b->plans[c].caTable : b->plans[c].vTable;
            auto key = std::make_pair(fnv(T.data.data(), T.data.size() * 8), T.data.size());
            auto it = tabDev.find(key);
            if (it == tabDev.end()) it = tabDev.emplace(key, b->buf.up(T.data, b->st)).first;
            (pass ? catab : vtab)[c] = it->second;
        }
    }
    // reinit arrays contiguous over cells
    size_t nInit = 0, nSyn = 0;
    b->initVmOff.resize(nC);
    b->synOff.resize(nC);
    for (uint32_t c = 0; c < nC; ++c) {
        b->initVmOff[c] = nInit;
        nInit += b->plans[c].N;
        b->synOff[c] = nSyn;
        nSyn += 5 * (size_t)b->plans[c].S;
    }
    b->dInitVm = b->buf.zeros<double>(nInit, b->st);
    b->dSynConst = b->buf.zeros<double>(nSyn, b->st);
    if (b->buf.err != cudaSuccess) return cerr(b->buf.err, "batch tables");
    std::vector<double> init(nInit);
    for (uint32_t c = 0; c < nC; ++c)
        std::copy(b->plans[c].initVm.begin(), b->plans[c].initVm.end(), init.begin() + b->initVmOff[c]);
    cudaError_t e = cudaMemcpyAsync(b->dInitVm, init.data(), nInit * 8, cudaMemcpyHostToDevice, b->st);
    if (e != cudaSuccess) return cerr(e, "batch initVm");
    // arena for all cells
    std::vector<CellShared> sh(nC);
    Arena dry;
    b->dcs.resize(nC);
    for (uint32_t c = 0; c < nC; ++c) {
        sh[c].initVm = b->dInitVm + b->initVmOff[c];
        sh[c].synConst = b->dSynConst + b->synOff[c];
        sh[c].vTab = vtab[c];
        sh[c].caTab = catab[c];
        sh[c].g2dBase = g2dBase;
        sh[c].g2dOff = g2dOffs[c];
        layoutCell(b->plans[c], dry, b->dcs[c], b->spikeCap, b->st, &sh[c]);
    }
    b->arena.size = dry.used + 256;
    e = cudaMalloc(&b->arena.base, b->arena.size);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->arena.base, 0, b->arena.size, b->st);
    for (uint32_t c = 0; c < nC && e == cudaSuccess; ++c)
        e = layoutCell(b->plans[c], b->arena, b->dcs[c], b->spikeCap, b->st, &sh[c]);
    if (e != cudaSuccess) return cerr(e, "batch upload");
    b->dDcs = b->buf.alloc<DevCell>(nC);
    if (b->buf.err != cudaSuccess) return cerr(b->buf.err, "batch cells");
    (void)cells;
    return HS_OK;
}

int uploadDcs(HsBatch* b) {
    for (DevCell& d : b->dcs) {
        d.dt = b->clockDt > 0 ? b->clockDt : b->dtSetup;
        d.caAdvance = b->caAdvance;
    }
    cudaError_t e = cudaMemcpyAsync(b->dDcs, b->dcs.data(), b->dcs.size() * sizeof(DevCell),
                                    cudaMemcpyHostToDevice, b->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
    return e == cudaSuccess ? HS_OK : cerr(e, "batch cell upload");
}

// ---- mixed batch --------------------------------------------------------------
template <class K>
int typeIndex(std::vector<K>& keys, const K& k, int maxTypes) {
    for (size_t i = 0; i < keys.size(); ++i)
        if (std::memcmp(&keys[i], &k, sizeof(K)) == 0) return (int)i;
    if ((int)keys.size() >= maxTypes) return -1;
    keys.push_back(k);
    return (int)keys.size() - 1;
}

int8_t powCode(double p, float& pf) {
    pf = (float)p;
    if (p == 0.0) return 0;
    if (p == 1.0) return 1;
    if (p == 2.0) return 2;
    if (p == 3.0) return 3;
    if (p == 4.0) return 4;
    return -1;
}

int buildMixed(HsBatch* b) {
    const uint32_t nC = b->nCells;
    MixHost& H = b->mh;
    // one shared V table and Ca table for the batch
    const Table& V0 = b->plans[0].vTable;
    const Table& C0 = b->plans[0].caTable;
    for (uint32_t c = 1; c < nC; ++c) {
        const Table& V = b->plans[c].vTable;
        const Table& Ca = b->plans[c].caTable;
        if (V.data != V0.data || V.min != V0.min || V.max != V0.max || Ca.data != C0.data)
            return berr(HS_ENOTSUP, "mixed batch: all cells must share one rate-table set");
    }
    std::vector<float> vtab(V0.data.begin(), V0.data.end()), catab(C0.data.begin(), C0.data.end());
    // 2-D tables by source identity, FP32 (A,B) interleaved
    std::map<std::tuple<const double*, const double*, uint32_t, uint32_t>, int> g2dIndex;
    std::vector<float> g2d, g2dGeom;
    std::vector<uint64_t> g2dOff;
    std::vector<uint32_t> g2dN;
    std::vector<ChanType> ctypes;
    std::vector<C2dType> ktypes;
    // node arrays
    std::vector<uint32_t> levelPtr, nodeInfo, child0, parent, chan0, state0, pool0, c2d0, syn0;
    std::vector<double> off, HS2, CmByDt, EmByRm, Vinit;
    std::vector<uint8_t> chanType, c2dType, synTypeV;
    std::vector<float> chanGbar, state, poolC, poolF1, poolF2, poolBasal, poolCeil, poolFloor, c2dGbar, c2dX;
    std::vector<uint32_t> injNode, stimStep, stimEntry, sgNode;
    std::vector<double> injVal, stimValue;
    std::vector<float> sgThresh, sgRefract;
    std::vector<int32_t> sgEdge;
    H.cells.resize(nC);
    H.nodeOf.resize(nC);
    H.poolOf.resize(nC);
    for (uint32_t ci = 0; ci < nC; ++ci) {
        const CellPlan& P = b->plans[ci];
        const uint32_t N = P.N;
        // star-form tree
        std::vector<int64_t> mparent(N, -1);
        for (uint32_t i = 0; i < N; ++i)
            for (uint32_t c : P.children[i]) mparent[c] = i;
        int64_t root = -1;
        for (uint32_t i = 0; i < N; ++i)
            if (mparent[i] < 0) root = i;
        std::vector<double> Ga(N), diag(N);
        for (uint32_t i = 0; i < N; ++i) {
            Ga[i] = 2.0 / P.Ra[i];
            diag[i] = P.Cm[i] / (P.dtSetup / 2.0) + 1.0 / P.Rm[i];
        }
        std::vector<std::vector<uint32_t>> tk(N);
        std::vector<double> toff(N, 0.0);
        for (uint32_t p = 0; p < N; ++p) {
            const std::vector<uint32_t>& ch = P.children[p];
            if (ch.size() == 1) {
                uint32_t c = ch[0];
                double g = Ga[p] * Ga[c] / (Ga[p] + Ga[c]);
                diag[p] += g;
                diag[c] += g;
                tk[p].push_back(c);
                toff[c] = -g;
            } else if (ch.size() >= 2) {
                uint32_t J = (uint32_t)diag.size();
                double gsum = Ga[p];
                for (uint32_t c : ch) gsum += Ga[c];
                diag.push_back(gsum);
                toff.push_back(-Ga[p]);
                tk.push_back(std::vector<uint32_t>(ch.begin(), ch.end()));
                diag[p] += Ga[p];
                tk[p].push_back(J);
                for (uint32_t c : ch) {
                    diag[c] += Ga[c];
                    toff[c] = -Ga[c];
                }
            }
        }
        const uint32_t T = (uint32_t)diag.size();
        // breadth-first order from the root
        std::vector<uint32_t> bfs;
        std::vector<uint32_t> level;
        bfs.reserve(T);
        bfs.push_back((uint32_t)root);
        std::vector<uint32_t> lvl(T, 0);
        for (size_t k = 0; k < bfs.size(); ++k)
            for (uint32_t c : tk[bfs[k]]) {
                lvl[c] = lvl[bfs[k]] + 1;
                bfs.push_back(c);
            }
        if (bfs.size() != T) return berr(HS_EINVAL, "mixed batch: tree construction failed");
        std::vector<uint32_t> pos(T);
        for (uint32_t k = 0; k < T; ++k) pos[bfs[k]] = k;
        MixCellRange& R = H.cells[ci];
        const uint32_t node0 = (uint32_t)nodeInfo.size();
        R.node0 = node0;
        R.nNodes = T;
        R.level0 = (uint32_t)levelPtr.size();
        uint32_t nL = lvl[bfs.back()] + 1;
        R.nLevels = nL;
        {
            std::vector<uint32_t> lp(nL + 1, 0);
            for (uint32_t k = 0; k < T; ++k) lp[lvl[bfs[k]] + 1]++;
            for (uint32_t l = 0; l < nL; ++l) lp[l + 1] += lp[l];
            levelPtr.insert(levelPtr.end(), lp.begin(), lp.end());
        }
        H.nodeOf[ci].assign(P.hinesOf.size(), -1);
        for (size_t m = 0; m < P.hinesOf.size(); ++m)
            if (P.hinesOf[m] >= 0) H.nodeOf[ci][m] = node0 + pos[P.hinesOf[m]];
        H.poolOf[ci].assign(P.poolSolverOf.size(), -1);
        // inject entries: basal injects and stimulus targets
        std::map<uint32_t, uint32_t> injEntry;   // compartment -> entry
        R.inj0 = (uint32_t)injNode.size();
        for (uint32_t i = 0; i < N; ++i)
            if (P.injPresent[i]) {
                injEntry[i] = (uint32_t)(injNode.size() - R.inj0);
                injNode.push_back(pos[i]);
                injVal.push_back(P.injBasal[i]);
            }
        for (uint32_t k = 0; k < P.stimCompt.size(); ++k)
            if (!injEntry.count(P.stimCompt[k])) {
                injEntry[P.stimCompt[k]] = (uint32_t)(injNode.size() - R.inj0);
                injNode.push_back(pos[P.stimCompt[k]]);
                injVal.push_back(0.0);
            }
        R.nInj = (uint32_t)injNode.size() - R.inj0;
        b->injEntryOf.emplace_back(P.hinesOf.size(), -1);
        for (auto& kv : injEntry) b->injEntryOf.back()[P.modelOf[kv.first]] = (int32_t)(R.inj0 + kv.second);
        R.stim0 = (uint32_t)stimStep.size();
        for (uint32_t k = 0; k < P.stimCompt.size(); ++k) {
            stimStep.push_back(P.stimStep[k]);
            stimEntry.push_back(injEntry[P.stimCompt[k]]);
            stimValue.push_back(P.stimValue[k]);
        }
        R.nStim = (uint32_t)stimStep.size() - R.stim0;
        R.sg0 = (uint32_t)sgNode.size();
        for (uint32_t k = 0; k < P.SG; ++k) {
            sgNode.push_back(pos[P.sgCompt[k]]);
            sgThresh.push_back((float)P.sgThreshold[k]);
            sgRefract.push_back((float)P.sgRefract[k]);
            sgEdge.push_back(P.sgEdge[k]);
        }
        R.nSg = P.SG;
        R.rec0 = 0;
        R.nRec = 0;
        // per compartment lists of external objects
        std::vector<std::vector<uint32_t>> c2dOf(N), synOf(N);
        for (uint32_t k = 0; k < P.K2; ++k) c2dOf[P.c2dCompt[k]].push_back(k);
        for (uint32_t k = 0; k < P.S; ++k) synOf[P.synCompt[k]].push_back(k);
        for (uint32_t k = 0; k < T; ++k) {
            const uint32_t t = bfs[k];
            const bool center = t >= N;
            uint32_t info = center ? kNodeCenter : 0;
            if (!center && injEntry.count(t)) info |= kNodeInject;
            nodeInfo.push_back(info);
            child0.push_back(0);    // filled below
            parent.push_back(0);
            off.push_back(toff[t]);
            HS2.push_back(diag[t]);
            CmByDt.push_back(center ? 0.0 : P.CmByDt[t]);
            EmByRm.push_back(center ? 0.0 : P.EmByRm[t]);
            Vinit.push_back(center ? 0.0 : P.initVm[t]);
            H.initVm.push_back(center ? 0.0 : P.initVm[t]);
            chan0.push_back((uint32_t)chanGbar.size());
            state0.push_back((uint32_t)state.size());
            pool0.push_back((uint32_t)poolC.size());
            c2d0.push_back((uint32_t)c2dGbar.size());
            syn0.push_back((uint32_t)synTypeV.size());
            if (center) continue;
            const uint32_t pb = P.poolPtr[t], pe = P.poolPtr[t + 1];
            if (pe - pb > 4) return berr(HS_ENOTSUP, "mixed batch: more than 4 Ca pools in a compartment");
            for (uint32_t p = pb; p < pe; ++p) {
                H.poolOf[ci][P.poolModel[p]] = (int64_t)poolC.size();
                poolC.push_back(0.f);
                poolF1.push_back((float)(1.0 - P.f1[p]));     // decay per step, in FP64
                poolF2.push_back((float)P.f2[p]);
                poolBasal.push_back((float)P.CaBasal[p]);
                poolCeil.push_back((float)P.ceiling[p]);
                poolFloor.push_back((float)P.floor_[p]);
            }
            for (uint32_t q = P.chanPtr[t]; q < P.chanPtr[t + 1]; ++q) {
                ChanType ty;
                std::memset(&ty, 0, sizeof(ty));
                ty.ek = (float)P.Ek[q];
                ty.xp = powCode(P.Xpow[q], ty.xpf);
                ty.yp = powCode(P.Ypow[q], ty.ypf);
                ty.zp = powCode(P.Zpow[q], ty.zpf);
                ty.instant = (int8_t)P.instant[q];
                ty.colX = (int16_t)(P.colX[q] < 0 ? 0 : P.colX[q]);
                ty.colY = (int16_t)(P.colY[q] < 0 ? 0 : P.colY[q]);
                ty.colZ = (int16_t)(P.colZ[q] < 0 ? 0 : P.colZ[q]);
                ty.zSrc = -1;
                if (P.Zpow[q] > 0.0 && P.zSrc[q] >= 0) {
                    if (P.zSrc[q] < (int32_t)pb || P.zSrc[q] >= (int32_t)pe)
                        return berr(HS_ENOTSUP, "mixed batch: Ca-dependent gate reads another compartment's pool");
                    ty.zSrc = (int8_t)(P.zSrc[q] - pb);
                }
                ty.caTarget = -1;
                if (P.caTarget[q] >= 0) {
                    if (P.caTarget[q] < (int32_t)pb || P.caTarget[q] >= (int32_t)pe)
                        return berr(HS_ENOTSUP, "mixed batch: channel feeds another compartment's pool");
                    ty.caTarget = (int8_t)(P.caTarget[q] - pb);
                }
                int ti = typeIndex(ctypes, ty, kMaxChanTypes);
                if (ti < 0) return berr(HS_ENOTSUP, "mixed batch: too many channel types");
                chanType.push_back((uint8_t)ti);
                chanGbar.push_back((float)(P.Gbar[q] * P.modulation[q]));
                int s = P.stateOff[q];
                if (P.Xpow[q] > 0.0) state.push_back((float)P.state0[s++]);
                if (P.Ypow[q] > 0.0) state.push_back((float)P.state0[s++]);
                if (P.Zpow[q] > 0.0) state.push_back((float)P.state0[s++]);
            }
            for (uint32_t k : c2dOf[t]) {
                const Gate2D& G = P.gates2d[P.c2dGate[k]];
                auto key = std::make_tuple(G.srcA, G.srcB, G.nx, G.ny);
                auto it = g2dIndex.find(key);
                if (it == g2dIndex.end()) {
                    if (g2dIndex.size() >= 127) return berr(HS_ENOTSUP, "mixed batch: too many 2-D tables");
                    int gi = (int)g2dN.size() / 2;
                    size_t n = (size_t)G.nx * G.ny;
                    g2dOff.push_back(g2d.size());
                    size_t o = g2d.size();
                    g2d.resize(o + 2 * n);
                    for (size_t i = 0; i < n; ++i) {
                        g2d[o + 2 * i] = (float)G.srcA[i];
                        g2d[o + 2 * i + 1] = (float)G.srcB[i];
                    }
                    g2dGeom.insert(g2dGeom.end(), {(float)G.xmin, (float)G.ymin, (float)G.invDx, (float)G.invDy,
                                                   (float)G.xmax, (float)G.ymax});
                    g2dN.push_back(G.nx);
                    g2dN.push_back(G.ny);
                    it = g2dIndex.emplace(key, gi).first;
                }
                C2dType ky;
                std::memset(&ky, 0, sizeof(ky));
                ky.ek = (float)P.c2dEk[k];
                ky.xp = powCode(P.c2dXpow[k], ky.xpf);
                ky.dep0 = (int8_t)P.c2dDep0[k];
                ky.dep1 = (int8_t)P.c2dDep1[k];
                ky.conc1 = -1;
                ky.conc2 = -1;
                if (P.c2dConc1[k] >= 0) {
                    if (P.c2dConc1[k] < (int32_t)pb || P.c2dConc1[k] >= (int32_t)pe)
                        return berr(HS_ENOTSUP, "mixed batch: HHChannel2D reads another compartment's pool");
                    ky.conc1 = (int8_t)(P.c2dConc1[k] - pb);
                }
                if (P.c2dConc2[k] >= 0) {
                    if (P.c2dConc2[k] < (int32_t)pb || P.c2dConc2[k] >= (int32_t)pe)
                        return berr(HS_ENOTSUP, "mixed batch: HHChannel2D reads another compartment's pool");
                    ky.conc2 = (int8_t)(P.c2dConc2[k] - pb);
                }
                ky.instant = (int8_t)P.c2dInstant[k];
                ky.gate = (int8_t)it->second;
                int ti = typeIndex(ktypes, ky, kMaxC2dTypes);
                if (ti < 0) return berr(HS_ENOTSUP, "mixed batch: too many HHChannel2D types");
                c2dType.push_back((uint8_t)ti);
                c2dGbar.push_back((float)(P.c2dGbar[k] * P.c2dMod[k]));
                c2dX.push_back((float)P.c2dX0[k]);
                H.c2dX0.push_back((float)P.c2dX0[k]);
            }
            for (uint32_t k : synOf[t]) {
                auto key = std::make_tuple(P.synTau1[k], P.synTau2[k], P.synEk[k]);
                size_t ti = 0;
                while (ti < H.synTypeKey.size() && H.synTypeKey[ti] != key) ++ti;
                if (ti == H.synTypeKey.size()) {
                    if (ti >= (size_t)kMaxSynTypes) return berr(HS_ENOTSUP, "mixed batch: too many SynChan types");
                    H.synTypeKey.push_back(key);
                }
                synTypeV.push_back((uint8_t)ti);
                H.synGbar.push_back(P.synGbar[k]);
                H.synTau1.push_back(P.synTau1[k]);
                H.synTau2.push_back(P.synTau2[k]);
                H.synMod.push_back(P.synMod[k]);
                H.evStart.push_back((uint32_t)H.evTime.size());
                for (uint32_t e = P.evPtr[k]; e < P.evPtr[k + 1]; ++e) {
                    H.evTime.push_back(P.evTime[e]);
                    H.evW.push_back(P.evW[e]);
                }
                H.evEnd.push_back((uint32_t)H.evTime.size());
            }
        }
        // children CSR and parents in global node indices
        {
            uint32_t next = node0 + 1;
            for (uint32_t k = 0; k < T; ++k) {
                child0[node0 + k] = next;
                for (uint32_t c : tk[bfs[k]]) parent[node0 + pos[c]] = node0 + k;
                next += (uint32_t)tk[bfs[k]].size();
            }
            parent[node0] = ~0u;
        }
    }
    // closing CSR entries
    const uint32_t nN = (uint32_t)nodeInfo.size();
    child0.push_back(nN);
    chan0.push_back((uint32_t)chanGbar.size());
    state0.push_back((uint32_t)state.size());
    pool0.push_back((uint32_t)poolC.size());
    c2d0.push_back((uint32_t)c2dGbar.size());
    syn0.push_back((uint32_t)synTypeV.size());
    H.nNodes = nN;
    // upload
    DevBuf& D = b->buf;
    cudaStream_t st = b->st;
    MixBatch& m = b->mb;
    std::memset(&m, 0, sizeof(m));
    m.nCells = nC;
    m.cells = D.up(H.cells, st);
    m.levelPtr = D.up(levelPtr, st);
    m.nodeInfo = D.up(nodeInfo, st);
    m.child0 = D.up(child0, st);
    m.parent = D.up(parent, st);
    m.off = D.up(off, st);
    m.HS2 = D.up(HS2, st);
    m.CmByDt = D.up(CmByDt, st);
    m.EmByRm = D.up(EmByRm, st);
    m.V = D.up(Vinit, st);
    m.VMid = D.zeros<double>(nN, st);
    m.rhsF = D.zeros<double>(nN, st);
    m.inv = D.zeros<double>(nN, st);
    m.chan0 = D.up(chan0, st);
    m.state0 = D.up(state0, st);
    m.pool0 = D.up(pool0, st);
    m.c2d0 = D.up(c2d0, st);
    m.syn0 = D.up(syn0, st);
    m.chanType = D.up(chanType, st);
    m.chanGbar = D.up(chanGbar, st);
    m.state = D.up(state, st);
    m.chanGk = D.zeros<float>(chanGbar.size(), st);
    m.poolC = D.up(poolC, st);
    m.poolCa = D.up(poolBasal, st);
    m.caG = D.zeros<float>(poolC.size(), st);
    m.caGE = D.zeros<float>(poolC.size(), st);
    m.poolF1 = D.up(poolF1, st);
    m.poolF2 = D.up(poolF2, st);
    m.poolBasal = D.up(poolBasal, st);
    m.poolCeil = D.up(poolCeil, st);
    m.poolFloor = D.up(poolFloor, st);
    m.c2dType = D.up(c2dType, st);
    m.c2dGbar = D.up(c2dGbar, st);
    m.c2dX = D.up(c2dX, st);
    m.g2d = D.up(g2d, st);
    m.g2dOff = D.up(g2dOff, st);
    m.g2dGeom = D.up(g2dGeom, st);
    m.g2dN = D.up(g2dN, st);
    m.synType = D.up(synTypeV, st);
    m.synX = D.zeros<float>(synTypeV.size(), st);
    m.synY = D.zeros<float>(synTypeV.size(), st);
    m.evCur = D.up(H.evStart, st);
    m.evEnd = D.up(H.evEnd, st);
    b->dEvStep = D.zeros<uint32_t>(H.evTime.size(), st);
    b->dEvAct = D.zeros<float>(H.evTime.size(), st);
    b->dSynNorm = D.zeros<float>(synTypeV.size(), st);
    m.evStep = b->dEvStep;
    m.evAct = b->dEvAct;
    m.synNorm = b->dSynNorm;
    m.injNode = D.up(injNode, st);
    m.injVal = D.up(injVal, st);
    m.stimStep = D.up(stimStep, st);
    m.stimEntry = D.up(stimEntry, st);
    m.stimValue = D.up(stimValue, st);
    m.stimCur = D.zeros<uint32_t>(nC, st);
    m.sgNode = D.up(sgNode, st);
    m.sgThresh = D.up(sgThresh, st);
    m.sgRefract = D.up(sgRefract, st);
    m.sgEdge = D.up(sgEdge, st);
    m.sgLast = D.zeros<float>(sgNode.size(), st);
    m.sgFired = D.zeros<int32_t>(sgNode.size(), st);
    m.spikeCap = b->spikeCap;
    m.spikeCount = D.zeros<uint32_t>(nC, st);
    m.spikeGen = D.zeros<uint32_t>((size_t)nC * b->spikeCap, st);
    m.spikeTime = D.zeros<float>((size_t)nC * b->spikeCap, st);
    m.vTab = D.up(vtab, st);
    m.vCol = V0.nCol;
    m.vRows = V0.nPts;
    m.vMin = (float)V0.min;
    m.vMax = (float)V0.max;
    m.vInvDx = (float)(1.0 / V0.dx);
    m.caTab = D.up(catab, st);
    m.caCol = C0.nCol;
    m.caRows = C0.nPts;
    m.caMin = (float)C0.min;
    m.caMax = (float)C0.max;
    m.caInvDx = C0.dx != 0.0 ? (float)(1.0 / C0.dx) : 0.f;
    m.recStride = 1;
    m.stepCount = D.zeros<unsigned long long>(nC, st);
    b->dMixInitVm = D.up(H.initVm, st);
    b->dMixC2dX0 = D.up(H.c2dX0, st);
    b->dEvStart = D.up(H.evStart, st);
    if (D.err != cudaSuccess) return cerr(D.err, "mixed batch upload");
    cudaError_t e = uploadMixedTypes(ctypes.data(), (int)ctypes.size(), ktypes.data(), (int)ktypes.size(),
                                     nullptr, 0, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cerr(e, "mixed batch types");
    return HS_OK;
}

}  // namespace

extern "C" {

int hs_batch_create(const HsCellDesc* cells, const uint32_t* seeds, uint32_t n_cells, double dt,
                    int precision, const HsBatchTuning* tuning, HsBatch** out) {
    if (!cells || !seeds || !out || n_cells == 0) return berr(HS_EINVAL, "bad batch arguments");
    *out = nullptr;
    if (precision != HS_PREC_FP64 && precision != HS_PREC_MIXED) return berr(HS_EINVAL, "unknown precision");
    HsBatch* b = new (std::nothrow) HsBatch();
    if (!b) return berr(HS_ENOMEM, "host allocation failed");
    b->precision = precision;
    b->nCells = n_cells;
    b->dtSetup = dt;
    b->plans.resize(n_cells);
    // set up every cell as HSolve::setup would (hs_plan.cpp), in parallel
    std::vector<std::string> errs(n_cells);
    std::vector<char> ok(n_cells, 0);
    {
        unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
        std::vector<std::thread> th;
        PlanOptions opt;
        opt.copyTables2d = false;
        for (unsigned t = 0; t < nt; ++t)
            th.emplace_back([&, t]() {
                for (uint32_t c = t; c < n_cells; c += nt) {
                    try {
                        ok[c] = buildPlan(cells[c], seeds[c], dt, b->plans[c], errs[c], opt);
                    } catch (...) {
                        errs[c] = "setup failed";
                    }
                }
            });
        for (auto& x : th) x.join();
    }
    for (uint32_t c = 0; c < n_cells; ++c)
        if (!ok[c]) {
            std::string m = "cell " + std::to_string(c) + ": " + errs[c];
            delete b;
            return berr(HS_EINVAL, m);
        }
    for (const CellPlan& P : b->plans) b->nCompt += P.N;
    int nd = 0;
    if (cudaGetDeviceCount(&nd) != cudaSuccess || nd == 0) {
        cudaGetLastError();
        delete b;
        return berr(HS_EDEVICE, "no CUDA device");
    }
    cudaError_t e = cudaGetDevice(&b->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->nSm, cudaDevAttrMultiProcessorCount, b->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete b;
        return cerr(e, "batch stream");
    }
    if (tuning) {
        if (tuning->threads_per_cta) b->threadsPerCta = tuning->threads_per_cta;
        if (tuning->ctas_per_sm) b->ctasPerSm = tuning->ctas_per_sm;
        if (tuning->steps_per_launch) b->stepsPerLaunch = tuning->steps_per_launch;
        b->useGraph = tuning->use_graph != 0;
    }
    if (b->threadsPerCta % 32 || b->threadsPerCta > 512 ||
        (precision == HS_PREC_FP64 && b->threadsPerCta > 256)) {
        hs_batch_destroy(b);
        return berr(HS_EINVAL, "threads_per_cta must be a multiple of 32, at most 512 (256 for FP64)");
    }
    int rc = precision == HS_PREC_FP64 ? buildFp64(b, cells) : buildMixed(b);
    if (rc == HS_OK && precision == HS_PREC_FP64) rc = uploadDcs(b);
    if (rc == HS_OK) rc = repack(b);
    if (rc != HS_OK) {
        std::string m = hs_last_error();
        hs_batch_destroy(b);
        return berr(rc, m);
    }
    *out = b;
    return HS_OK;
}

int hs_batch_destroy(HsBatch* b) {
    if (!b) return HS_OK;
    if (b->st) cudaStreamSynchronize(b->st);
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    for (auto& p : b->evs) {
        cudaEventDestroy(p.first);
        cudaEventDestroy(p.second);
    }
    b->buf.freeAll();
    b->packBuf.freeAll();
    b->recBuf.freeAll();
    b->injBuf.freeAll();
    if (b->arena.base) cudaFree(b->arena.base);
    if (b->st) cudaStreamDestroy(b->st);
    delete b;
    return HS_OK;
}

int hs_batch_tune(HsBatch* b, const HsBatchTuning* t) {
    if (!b || !t) return berr(HS_EINVAL, "null argument");
    if (t->threads_per_cta) {
        if (t->threads_per_cta % 32 || t->threads_per_cta > 512)
            return berr(HS_EINVAL, "threads_per_cta must be a multiple of 32, at most 512");
        b->threadsPerCta = t->threads_per_cta;
    }
    if (t->ctas_per_sm) b->ctasPerSm = t->ctas_per_sm;
    if (t->steps_per_launch) b->stepsPerLaunch = t->steps_per_launch;
    b->useGraph = t->use_graph != 0;
    cudaStreamSynchronize(b->st);
    return repack(b);
}

int hs_batch_reinit(HsBatch* b, double clock_dt) {
    if (!b) return berr(HS_EINVAL, "null batch");
    if (!(clock_dt > 0)) return berr(HS_EINVAL, "clock dt must be positive");
    if (b->gexec) {
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
    }
    b->clockDt = clock_dt;
    b->stepsDone = 0;
    cudaError_t e = cudaSuccess;
    if (b->precision == HS_PREC_FP64) {
        size_t nsc = b->synOff.back() + 5 * (size_t)b->plans.back().S;
        std::vector<double> sc(nsc + 1);
        for (uint32_t c = 0; c < b->nCells; ++c) synConsts(b->plans[c], clock_dt, sc.data() + b->synOff[c]);
        if (nsc) e = cudaMemcpyAsync(b->dSynConst, sc.data(), nsc * 8, cudaMemcpyHostToDevice, b->st);
        if (e != cudaSuccess) return cerr(e, "batch reinit");
        int rc = uploadDcs(b);
        if (rc) return rc;
        e = launchReinitFp64(b->dDcs, b->nCells, b->st);
    } else {
        MixHost& H = b->mh;
        // SynChan constants and event delivery steps at the clock dt
        std::vector<SynType> types(H.synTypeKey.size());
        for (size_t t = 0; t < types.size(); ++t) {
            double xc1, xc2, yc1, yc2, norm;
            synchanConstants(std::get<0>(H.synTypeKey[t]), std::get<1>(H.synTypeKey[t]), 1.0, clock_dt, &xc1,
                             &xc2, &yc1, &yc2, &norm);
            types[t] = {(float)xc1, (float)xc2, (float)yc1, (float)yc2, (float)std::get<2>(H.synTypeKey[t])};
        }
        std::vector<float> norm(H.synGbar.size());
        for (size_t k = 0; k < norm.size(); ++k) {
            double xc1, xc2, yc1, yc2, nm;
            synchanConstants(H.synTau1[k], H.synTau2[k], H.synGbar[k], clock_dt, &xc1, &xc2, &yc1, &yc2, &nm);
            norm[k] = (float)(nm * H.synMod[k]);
        }
        std::vector<uint32_t> evStep(H.evTime.size());
        std::vector<float> evAct(H.evTime.size());
        for (size_t e2 = 0; e2 < H.evTime.size(); ++e2) {
            // first step whose currTime = dt * (step + 1) reaches the event
            // time (SimpleSynHandler delivers events with time <= currTime)
            double t = H.evTime[e2];
            double g = std::ceil(t / clock_dt) - 3.0;
            uint64_t s = g > 0 ? (uint64_t)g : 0;
            while (!(t <= clock_dt * (double)(s + 1))) ++s;
            evStep[e2] = (uint32_t)std::min<uint64_t>(s, 0xffffffffu);
            evAct[e2] = (float)(H.evW[e2] / clock_dt);
        }
        e = uploadMixedTypes(nullptr, 0, nullptr, 0, types.data(), (int)types.size(), b->st);
        if (e == cudaSuccess && !norm.empty())
            e = cudaMemcpyAsync(b->dSynNorm, norm.data(), norm.size() * 4, cudaMemcpyHostToDevice, b->st);
        if (e == cudaSuccess && !evStep.empty())
            e = cudaMemcpyAsync(b->dEvStep, evStep.data(), evStep.size() * 4, cudaMemcpyHostToDevice, b->st);
        if (e == cudaSuccess && !evAct.empty())
            e = cudaMemcpyAsync(b->dEvAct, evAct.data(), evAct.size() * 4, cudaMemcpyHostToDevice, b->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);   // host vectors go out of scope
        b->mb.dt = clock_dt;
        b->mb.dtf = (float)clock_dt;
        b->mb.caAdvance = b->caAdvance;
        if (e == cudaSuccess) e = launchBatchReinitMixed(b->mb, b->dMixInitVm, b->dMixC2dX0, b->dEvStart, b->st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
    if (e != cudaSuccess) return cerr(e, "batch reinit");
    b->reinited = true;
    return HS_OK;
}

int hs_batch_process(HsBatch* b, uint32_t nsteps) {
    if (!b) return berr(HS_EINVAL, "null batch");
    if (!b->reinited) return berr(HS_ESTATE, "reinit before process");
    if (nsteps == 0) return HS_OK;
    const uint32_t K = b->stepsPerLaunch;
    auto timedLaunch = [&](uint32_t k) -> cudaError_t {
        if (b->evUsed == b->evs.size()) {
            cudaEvent_t a, z;
            cudaEventCreate(&a);
            cudaEventCreate(&z);
            b->evs.push_back({a, z});
        }
        auto& pr = b->evs[b->evUsed++];
        cudaEventRecord(pr.first, b->st);
        cudaError_t e = launchStep(b, k);
        cudaEventRecord(pr.second, b->st);
        return e;
    };
    cudaError_t e = cudaSuccess;
    if (b->useGraph && nsteps >= K) {
        // one graph for the full multiples of K; rebuilt when nsteps changes
        uint32_t full = nsteps / K * K;
        if (!b->gexec || b->gSteps != full) {
            if (b->gexec) cudaGraphExecDestroy(b->gexec);
            b->gexec = nullptr;
            cudaGraph_t g;
            e = cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal);
            for (uint32_t s = 0; s < full && e == cudaSuccess; s += K) e = launchStep(b, K);
            cudaError_t e2 = cudaStreamEndCapture(b->st, &g);
            if (e == cudaSuccess) e = e2;
            if (e == cudaSuccess) e = cudaGraphInstantiate(&b->gexec, g, 0);
            if (e2 == cudaSuccess) cudaGraphDestroy(g);
            b->gSteps = full;
        }
        if (b->evUsed == b->evs.size()) {
            cudaEvent_t a, z;
            cudaEventCreate(&a);
            cudaEventCreate(&z);
            b->evs.push_back({a, z});
        }
        auto& pr = b->evs[b->evUsed++];
        if (e == cudaSuccess) e = cudaEventRecord(pr.first, b->st);
        if (e == cudaSuccess) e = cudaGraphLaunch(b->gexec, b->st);
        if (e == cudaSuccess) e = cudaEventRecord(pr.second, b->st);
        b->timedLaunches += full / K - 1;     // the pair spans full/K launches
        if (e == cudaSuccess && nsteps > full) e = timedLaunch(nsteps - full);
    } else {
        for (uint32_t s = 0; s < nsteps && e == cudaSuccess; s += K) e = timedLaunch(std::min(K, nsteps - s));
    }
    if (e != cudaSuccess) return cerr(e, "batch process");
    b->stepsDone += nsteps;
    return HS_OK;
}

int hs_batch_sync(HsBatch* b) {
    if (!b) return berr(HS_EINVAL, "null batch");
    cudaError_t e = cudaStreamSynchronize(b->st);
    return e == cudaSuccess ? HS_OK : cerr(e, "batch sync");
}

int hs_batch_kernel_time(HsBatch* b, double* avg_ms, uint32_t* launches) {
    if (!b || !avg_ms || !launches) return berr(HS_EINVAL, "null argument");
    cudaError_t e = cudaStreamSynchronize(b->st);
    if (e != cudaSuccess) return cerr(e, "kernel time");
    for (size_t i = 0; i < b->evUsed; ++i) {
        float ms = 0;
        cudaEventElapsedTime(&ms, b->evs[i].first, b->evs[i].second);
        b->timedMs += ms;
        b->timedLaunches += 1;
    }
    b->evUsed = 0;
    *launches = b->timedLaunches;
    *avg_ms = b->timedLaunches ? b->timedMs / b->timedLaunches : 0.0;
    b->timedMs = 0;
    b->timedLaunches = 0;
    return HS_OK;
}

int hs_batch_stream(HsBatch* b, void** stream) {
    if (!b || !stream) return berr(HS_EINVAL, "null argument");
    *stream = (void*)b->st;
    return HS_OK;
}

int hs_batch_info(HsBatch* b, uint64_t* n_compt, uint32_t* n_ctas, uint32_t* threads_per_cta,
                  uint32_t* steps_per_launch) {
    if (!b) return berr(HS_EINVAL, "null batch");
    if (n_compt) *n_compt = b->nCompt;
    if (n_ctas) *n_ctas = b->nCtas;
    if (threads_per_cta) *threads_per_cta = b->threadsPerCta;
    if (steps_per_launch) *steps_per_launch = b->stepsPerLaunch;
    return HS_OK;
}

int hs_batch_read_vm(HsBatch* b, uint32_t cell, double* out, uint32_t n) {
    if (!b || !out) return berr(HS_EINVAL, "null argument");
    if (cell >= b->nCells) return berr(HS_EINVAL, "cell index out of range");
    const CellPlan& P = b->plans[cell];
    if (n != P.hinesOf.size()) return berr(HS_EINVAL, "n must equal the cell's compartment count");
    cudaError_t e = cudaStreamSynchronize(b->st);
    if (b->precision == HS_PREC_FP64) {
        std::vector<double> v(P.N);
        if (e == cudaSuccess) e = cudaMemcpy(v.data(), b->dcs[cell].V, P.N * 8, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cerr(e, "batch read vm");
        for (uint32_t m = 0; m < n; ++m) out[m] = P.hinesOf[m] < 0 ? NAN : v[P.hinesOf[m]];
    } else {
        const MixCellRange& R = b->mh.cells[cell];
        std::vector<double> v(R.nNodes);
        if (e == cudaSuccess) e = cudaMemcpy(v.data(), b->mb.V + R.node0, R.nNodes * 8, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cerr(e, "batch read vm");
        for (uint32_t m = 0; m < n; ++m) {
            int64_t g = b->mh.nodeOf[cell][m];
            out[m] = g < 0 ? NAN : v[g - R.node0];
        }
    }
    return HS_OK;
}

int hs_batch_read_ca(HsBatch* b, uint32_t cell, double* out, uint32_t n) {
    if (!b || !out) return berr(HS_EINVAL, "null argument");
    if (cell >= b->nCells) return berr(HS_EINVAL, "cell index out of range");
    const CellPlan& P = b->plans[cell];
    if (n != P.poolSolverOf.size()) return berr(HS_EINVAL, "n must equal the cell's pool count");
    cudaError_t e = cudaStreamSynchronize(b->st);
    if (e != cudaSuccess) return cerr(e, "batch read ca");
    if (b->precision == HS_PREC_FP64) {
        std::vector<double> v(P.P + 1);
        if (P.P) e = cudaMemcpy(v.data(), b->dcs[cell].ca, P.P * 8, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cerr(e, "batch read ca");
        for (uint32_t m = 0; m < n; ++m) out[m] = P.poolSolverOf[m] < 0 ? NAN : v[P.poolSolverOf[m]];
    } else {
        for (uint32_t m = 0; m < n; ++m) {
            int64_t g = b->mh.poolOf[cell][m];
            float x = NAN;
            if (g >= 0) e = cudaMemcpy(&x, b->mb.poolCa + g, 4, cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) return cerr(e, "batch read ca");
            out[m] = g < 0 ? NAN : x;
        }
    }
    return HS_OK;
}

int hs_batch_record(HsBatch* b, const uint32_t* cell, const uint32_t* compt, uint32_t n, uint32_t stride,
                    uint32_t capacity) {
    if (!b) return berr(HS_EINVAL, "null batch");
    if (n && (!cell || !compt || stride == 0 || capacity == 0)) return berr(HS_EINVAL, "bad recording request");
    cudaStreamSynchronize(b->st);
    if (b->gexec) {
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
    }
    b->recBuf.freeAll();
    b->recBuf.err = cudaSuccess;
    b->rec.clear();
    // group by cell, keep the request order within a cell
    std::vector<std::vector<uint32_t>> per(b->nCells);
    for (uint32_t r = 0; r < n; ++r) {
        if (cell[r] >= b->nCells) return berr(HS_EINVAL, "recorded cell out of range");
        const CellPlan& P = b->plans[cell[r]];
        if (compt[r] >= P.hinesOf.size() || P.hinesOf[compt[r]] < 0)
            return berr(HS_EINVAL, "recorded compartment not in the cell");
        per[cell[r]].push_back(compt[r]);
    }
    b->recCap = capacity;
    b->recStride = stride;
    double* buf = n ? b->recBuf.zeros<double>((size_t)n * capacity, b->st) : nullptr;
    b->recBase = buf;
    uint32_t col = 0;
    if (b->precision == HS_PREC_FP64) {
        std::vector<uint32_t> hidx;
        std::vector<uint32_t> starts(b->nCells);
        for (uint32_t c = 0; c < b->nCells; ++c) {
            starts[c] = (uint32_t)hidx.size();
            for (uint32_t m : per[c]) {
                hidx.push_back((uint32_t)b->plans[c].hinesOf[m]);
                b->rec.push_back({c, m});
            }
        }
        uint32_t* didx = b->recBuf.up(hidx, b->st);
        for (uint32_t c = 0; c < b->nCells; ++c) {
            DevCell& d = b->dcs[c];
            d.nRec = (uint32_t)per[c].size();
            d.recStride = stride;
            d.recCap = capacity;
            d.recLd = n;
            d.recCompt = didx + starts[c];
            d.recBuf = buf + starts[c];
        }
        if (b->recBuf.err != cudaSuccess) return cerr(b->recBuf.err, "batch record");
        return uploadDcs(b);
    }
    std::vector<uint32_t> nodes;
    for (uint32_t c = 0; c < b->nCells; ++c) {
        MixCellRange& R = b->mh.cells[c];
        R.rec0 = col;
        R.nRec = (uint32_t)per[c].size();
        for (uint32_t m : per[c]) {
            nodes.push_back((uint32_t)(b->mh.nodeOf[c][m] - R.node0));
            b->rec.push_back({c, m});
        }
        col += R.nRec;
    }
    b->mb.recNode = b->recBuf.up(nodes, b->st);
    b->mb.recBuf = buf;
    b->mb.recLd = n;
    b->mb.recCap = capacity;
    b->mb.recStride = stride;
    cudaError_t e = b->recBuf.err;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync((void*)b->mb.cells, b->mh.cells.data(), b->mh.cells.size() * sizeof(MixCellRange),
                            cudaMemcpyHostToDevice, b->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
    return e == cudaSuccess ? HS_OK : cerr(e, "batch record");
}

int hs_batch_read_trace(HsBatch* b, double* out, uint32_t capacity, uint32_t* n_samples) {
    if (!b || !n_samples) return berr(HS_EINVAL, "null argument");
    cudaError_t e = cudaStreamSynchronize(b->st);
    if (e != cudaSuccess) return cerr(e, "batch trace");
    uint64_t produced = b->rec.empty() ? 0 : b->stepsDone / b->recStride + 1;
    *n_samples = (uint32_t)produced;
    uint32_t stored = (uint32_t)std::min<uint64_t>(produced, b->recCap);
    uint32_t k = std::min(stored, capacity);
    if (out && k && !b->rec.empty()) {
        e = cudaMemcpy(out, b->recBase, (size_t)k * b->rec.size() * 8, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cerr(e, "batch trace");
    }
    return HS_OK;
}

int hs_batch_read_trace_window(HsBatch* b, uint32_t first, uint32_t count, double* out) {
    if (!b || (!out && count)) return berr(HS_EINVAL, "null argument");
    if (b->rec.empty()) return berr(HS_ESTATE, "nothing is recorded");
    if ((uint64_t)first + count > b->recCap) return berr(HS_ECAPACITY, "window beyond the recording capacity");
    if (!count) return HS_OK;
    cudaError_t e = cudaMemcpyAsync(out, b->recBase + (size_t)first * b->rec.size(),
                                    (size_t)count * b->rec.size() * 8, cudaMemcpyDeviceToHost, b->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
    return e == cudaSuccess ? HS_OK : cerr(e, "trace window");
}

int hs_batch_inject_targets(HsBatch* b, const uint32_t* cell, const uint32_t* compt, uint32_t n) {
    if (!b || (n && (!cell || !compt))) return berr(HS_EINVAL, "null argument");
    std::vector<double*> addr(n);
    std::vector<uint8_t*> flag(n, nullptr);
    for (uint32_t k = 0; k < n; ++k) {
        if (cell[k] >= b->nCells) return berr(HS_EINVAL, "inject target cell out of range");
        const CellPlan& P = b->plans[cell[k]];
        if (compt[k] >= P.hinesOf.size() || P.hinesOf[compt[k]] < 0)
            return berr(HS_EINVAL, "inject target compartment not in the cell");
        if (b->precision == HS_PREC_FP64) {
            uint32_t h = (uint32_t)P.hinesOf[compt[k]];
            addr[k] = b->dcs[cell[k]].injBasal + h;
            flag[k] = b->dcs[cell[k]].injPresent + h;
        } else {
            int32_t e = b->injEntryOf[cell[k]][compt[k]];
            if (e < 0)
                return berr(HS_ENOTSUP, "mixed batch: compartment had no inject or stimulus at setup");
            addr[k] = b->mb.injVal + e;
        }
    }
    cudaStreamSynchronize(b->st);
    b->injBuf.freeAll();
    b->injBuf.err = cudaSuccess;
    b->dInjAddr = b->injBuf.up(addr, b->st);
    b->dInjFlag = b->injBuf.up(flag, b->st);
    b->dInjVal = b->injBuf.alloc<double>(n);
    if (b->injBuf.err == cudaSuccess) b->injBuf.err = cudaStreamSynchronize(b->st);
    if (b->injBuf.err != cudaSuccess) return cerr(b->injBuf.err, "inject targets");
    b->nInjTargets = n;
    return HS_OK;
}

int hs_batch_set_inject(HsBatch* b, const double* values, uint32_t n) {
    if (!b || (n && !values)) return berr(HS_EINVAL, "null argument");
    if (n != b->nInjTargets) return berr(HS_EINVAL, "n must equal the registered target count");
    cudaError_t e = cudaMemcpyAsync(b->dInjVal, values, (size_t)n * 8, cudaMemcpyHostToDevice, b->st);
    if (e == cudaSuccess) e = launchScatterInject(b->dInjAddr, b->dInjFlag, b->dInjVal, n, b->st);
    return e == cudaSuccess ? HS_OK : cerr(e, "set inject");
}

int hs_batch_read_spikes(HsBatch* b, uint32_t* cell, uint32_t* gen, double* time, uint32_t capacity,
                         uint32_t* n) {
    if (!b || !n) return berr(HS_EINVAL, "null argument");
    cudaError_t e = cudaStreamSynchronize(b->st);
    if (e != cudaSuccess) return cerr(e, "batch spikes");
    uint32_t total = 0, k = 0;
    bool overflow = false;
    if (b->precision == HS_PREC_FP64) {
        for (uint32_t c = 0; c < b->nCells; ++c) {
            DevCtl ctl;
            e = cudaMemcpy(&ctl, b->dcs[c].ctl, sizeof(ctl), cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) return cerr(e, "batch spikes");
            uint32_t m = std::min(ctl.nSpikes, b->dcs[c].spikeCap);
            overflow |= ctl.nSpikes > m;
            total += ctl.nSpikes;
            if (!m || k >= capacity) continue;
            std::vector<uint32_t> g(m);
            std::vector<double> t(m);
            cudaMemcpy(g.data(), b->dcs[c].spikeGen, m * 4, cudaMemcpyDeviceToHost);
            cudaMemcpy(t.data(), b->dcs[c].spikeTime, m * 8, cudaMemcpyDeviceToHost);
            for (uint32_t i = 0; i < m && k < capacity; ++i, ++k) {
                if (cell) cell[k] = c;
                if (gen) gen[k] = g[i];
                if (time) time[k] = t[i];
            }
        }
    } else {
        std::vector<uint32_t> cnt(b->nCells);
        e = cudaMemcpy(cnt.data(), b->mb.spikeCount, b->nCells * 4, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cerr(e, "batch spikes");
        for (uint32_t c = 0; c < b->nCells; ++c) {
            uint32_t m = std::min(cnt[c], b->spikeCap);
            overflow |= cnt[c] > m;
            total += cnt[c];
            if (!m || k >= capacity) continue;
            std::vector<uint32_t> g(m);
            std::vector<float> t(m);
            cudaMemcpy(g.data(), b->mb.spikeGen + (size_t)c * b->spikeCap, m * 4, cudaMemcpyDeviceToHost);
            cudaMemcpy(t.data(), b->mb.spikeTime + (size_t)c * b->spikeCap, m * 4, cudaMemcpyDeviceToHost);
            for (uint32_t i = 0; i < m && k < capacity; ++i, ++k) {
                if (cell) cell[k] = c;
                if (gen) gen[k] = g[i];
                if (time) time[k] = t[i];
            }
        }
    }
    *n = total;
    if (overflow) return berr(HS_ECAPACITY, "a cell's spike buffer overflowed");
    return HS_OK;
}

}  // extern "C"
