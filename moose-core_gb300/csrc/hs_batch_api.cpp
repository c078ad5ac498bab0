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
#include "hs_events.h"
#include "hs_mixed.cuh"
#include "hs_noalloc.h"
#include "hs_plan.h"

namespace hsg {
int setLastError(int code, const std::string& msg);
cudaError_t launchForestStepMixed(const MixBatch& b, const uint32_t* ctaPtr, const uint32_t* ctaForests,
                                  uint32_t nCtas, uint32_t threadsPerCta, uint32_t smemBytes, uint32_t cap,
                                  uint32_t elimWarps, uint32_t nsteps, cudaStream_t st);
cudaError_t launchForestStepMixedCluster(const MixBatch& b, const uint32_t* ctaPtr, const uint32_t* ctaForests,
                                         uint32_t nClusters, uint32_t kC, uint32_t threadsPerCta,
                                         uint32_t smemBytes, uint32_t cap, uint32_t stageCap, uint32_t elimWarps,
                                         uint32_t nsteps, cudaStream_t st);
cudaError_t launchBatchReinitMixed(const MixBatch& b, uint32_t nNodes, const double* initVm, const float* c2dX0,
                                   const uint32_t* evStart, cudaStream_t st);
cudaError_t launchScatterInject(double* const* addr, uint8_t* const* flag, const double* val, uint32_t n,
                                cudaStream_t st);
cudaError_t launchScatterValues(const ValueWrite* w, uint32_t n, cudaStream_t st);
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

// Device buffers allocated and freed in stream order on the batch's stream
// (cudaMallocAsync / cudaFreeAsync from the device's pool): unlike cudaFree,
// releasing a batch does not wait for the work of other batches running on
// the GPU.
struct DevBuf {
    std::vector<void*> ptrs;
    cudaError_t err = cudaSuccess;
    uint64_t bytes = 0;
    cudaStream_t st = nullptr;
    template <class T>
    T* alloc(size_t n) {
        void* p = nullptr;
        if (err == cudaSuccess) err = cudaMallocAsync(&p, (n ? n : 1) * sizeof(T), st);
        if (err == cudaSuccess) {
            ptrs.push_back(p);
            bytes += (n ? n : 1) * sizeof(T);
        }
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
        for (void* p : ptrs) cudaFreeAsync(p, st);
        ptrs.clear();
        bytes = 0;
    }
};

// Host mirror of the mixed layout needed after creation.
struct MixHost {
    std::vector<MixCellRange> cells;
    std::vector<std::vector<int64_t>> nodeOf;     // per cell: model compartment -> global node
    std::vector<std::vector<int64_t>> poolOf;     // per cell: model pool -> global pool
    std::vector<std::vector<int64_t>> chanSlot;   // per cell: model HHChannel -> node * kMaxChan + slot
    std::vector<std::vector<int64_t>> c2dNode;    // per cell: model HHChannel2D -> node
    std::vector<std::vector<int64_t>> synGlobal;  // per cell: model SynChan -> global SynChan
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
    uint32_t nForests = 0, nShared = 0;           // forests, of them in shared memory
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
    // FP64 default: 4 CTAs of 128 threads per SM, the launch shape measured
    // fastest on the 4,096-cell workload (bit-identical in every shape)
    uint32_t threadsPerCta = 128, ctasPerSm = 4, stepsPerLaunch = 100;
    uint32_t forestNodes = 0;    // mixed: forest size limit (0: shared-memory capacity)
    uint32_t maxCtas = 0;        // mixed: CTA limit of the packing (0: one wave)
    uint32_t clusterCtas = 1;    // mixed: CTAs per forest group (2..8: a thread-block cluster)
    uint32_t mixStageCap = 0;    // mixed, clusters: largest forest whose OFF/TOPO/PAR rank 0 stages
    uint32_t elimWarps = 4;      // mixed: eliminator warps of the split step (0: no split)
    uint32_t waitRounds = 1u << 24;   // mixed: sleep rounds of one bounded wait (~128 ns each)
    bool useGraph = true;
    uint32_t nWarps = 0, nCtas = 0;
    uint32_t *dWarpPtr = nullptr, *dWarpCells = nullptr;
    uint32_t *dCtaCellPtr = nullptr, *dCtaCells = nullptr;   // FP64: cells stepped by a whole CTA
    uint32_t nCtaWhole = 0;
    // mixed: forests per CTA, shared-memory forest capacity
    uint32_t *dCtaPtr = nullptr, *dCtaForests = nullptr;
    uint32_t mixCap = 0, mixSmem = 0;
    unsigned long long* dStopStep = nullptr;    // mixed: per-cell stop steps
    unsigned long long* dForestStop = nullptr;  // mixed: per-forest largest stop step
    std::vector<uint32_t> forestCellPtr, forestCellIdx;   // mixed: cells of each forest (host)
    SynType* dSynTypes = nullptr;               // mixed: SynChan constants at the clock dt
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
    uint32_t* dEvCurDesc = nullptr;            // the description's cursors and ends
    const uint32_t* dEvEndDesc = nullptr;
    // run-time synaptic events (hs_batch_push_events): pushes wait on the
    // host, by global SynChan, until the next process call; the first flush
    // replaces the description's queues by a batch-owned queue over every
    // SynChan (global order: FP64 cell-major, mixed forest order) holding
    // the undelivered events, mirrored on the host
    std::vector<uint32_t> pendSyn;
    std::vector<double> pendTime, pendW;
    bool evOwned = false;
    std::vector<uint32_t> evHostPtr;           // S+1 starts of the owned queue
    std::vector<double> evHostTime, evHostW;
    uint32_t* dEvOwnCur = nullptr;             // cursors of the owned queue
    DevBuf evBuf;
    std::vector<uint32_t> synBase;             // FP64: first global SynChan of each cell
    struct EvPtrs {
        const uint32_t* ptr;
        uint32_t* cur;
        const double *time, *w;
    };
    std::vector<EvPtrs> evDesc;                // FP64: each cell's description queue
    // recording
    std::vector<std::pair<uint32_t, uint32_t>> rec;
    DevBuf recBuf;
    double* recBase = nullptr;
    uint32_t recCap = 0, recStride = 1;
    // bulk reads of every cell (hs_batch_read_all): gather lists built on
    // first use, dropped with the layout
    DevBuf gatherBuf;
    const void** dGatherVm = nullptr;
    const void** dGatherCa = nullptr;
    double* dGatherOut = nullptr;
    uint64_t nAllCompt = 0, nAllPool = 0;
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
        return launchBatchStepFp64(b->dDcs, b->dWarpPtr, b->dWarpCells, b->nWarps, b->dCtaCellPtr, b->dCtaCells, k,
                                   b->threadsPerCta, b->st);
    const uint32_t ew = b->elimWarps && b->threadsPerCta > 32 * b->elimWarps ? b->elimWarps : 0;
    b->mb.waitRounds = b->waitRounds;
    if (b->clusterCtas > 1) {
        // every forest is in global memory: twice the eliminator warps, as
        // the one-CTA serving kernel gives its global forests
        const uint32_t ce = std::min<uint32_t>(2 * (ew ? ew : 4), std::min<uint32_t>(16, b->threadsPerCta / 64));
        return launchForestStepMixedCluster(b->mb, b->dCtaPtr, b->dCtaForests, b->nCtas, b->clusterCtas,
                                            b->threadsPerCta, b->mixSmem, b->mixCap, b->mixStageCap, ce, k,
                                            b->st);
    }
    return launchForestStepMixed(b->mb, b->dCtaPtr, b->dCtaForests, b->nCtas, b->threadsPerCta, b->mixSmem,
                                 b->mixCap, ew, k, b->st);
}

// Packing of the FP64 batch into one wave of CTAs (as many per SM as the
// kernel's registers allow, at most ctas_per_sm).  A warp steps its cells
// one after the other, so a cell costing more than the balanced load of one
// warp would bound the step by itself: such cells are stepped by a whole
// CTA instead (its warps share each compartment loop and each elimination
// level, as in the drop-in), packed longest first over enough CTAs to carry
// their load; the other cells are packed longest first over the remaining
// CTAs and then over their warps.
int repack(HsBatch* b) {
    if (b->gexec) {
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
    }
    if (b->precision != HS_PREC_FP64) return HS_OK;
    b->packBuf.freeAll();
    b->packBuf.err = cudaSuccess;
    const uint32_t warpsPerCta = b->threadsPerCta / 32;
    const int fit = fp64BatchCtasPerSm(b->threadsPerCta);
    const uint32_t cps = std::max<uint32_t>(1, fit > 0 ? std::min<uint32_t>(b->ctasPerSm, (uint32_t)fit) : b->ctasPerSm);
    b->nCtas = std::max<uint32_t>(1, b->nSm * cps);
    b->nWarps = b->nCtas * warpsPerCta;
    std::vector<double> cost(b->nCells);
    double total = 0;
    for (uint32_t c = 0; c < b->nCells; ++c) {
        const CellPlan& P = b->plans[c];
        cost[c] = P.N + 0.3 * P.C + 0.5 * P.S + 2.0 * (P.fLevelPtr.size() + P.bLevelPtr.size());
        total += cost[c];
    }
    std::vector<uint32_t> order(b->nCells);
    for (uint32_t c = 0; c < b->nCells; ++c) order[c] = c;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) { return cost[x] > cost[y]; });
    // a whole CTA steps a cell at a fraction of its warps' combined rate
    // (a barrier per elimination level, levels narrower than the CTA); this
    // estimate of the fraction only decides which cells get whole CTAs
    constexpr double kCtaEfficiency = 0.6;
    const double ctaRate = warpsPerCta > 1 ? warpsPerCta * kCtaEfficiency : 1.0;
    // the k costliest cells on m whole CTAs, the rest over the warps of the
    // other CTAs: estimated step time, the larger of the two groups' (each
    // bounded below by its largest cell and by its load spread evenly)
    const uint32_t nC = b->nCells;
    std::vector<double> prefix(nC + 1, 0.0);
    for (uint32_t i = 0; i < nC; ++i) prefix[i + 1] = prefix[i] + cost[order[i]];
    uint32_t bestK = 0, bestM = 0;
    double bestT = std::max(nC ? cost[order[0]] : 0.0, total / b->nWarps);
    if (warpsPerCta > 1 && b->nCtas > 1)
        for (uint32_t k = 1; k <= nC; ++k) {
            const double sb = prefix[k], ss = total - sb;
            const double bigMax = cost[order[0]] / ctaRate, smallMax = k < nC ? cost[order[k]] : 0.0;
            // m balancing sb / (m ctaRate) against ss / ((nCtas - m) warpsPerCta)
            const double mf = k < nC ? b->nCtas * sb / ctaRate / (sb / ctaRate + ss / warpsPerCta) : b->nCtas;
            for (int dm = 0; dm <= 1; ++dm) {
                uint32_t m = (uint32_t)std::floor(mf) + dm;
                m = std::max<uint32_t>(1, std::min<uint32_t>(m, k < nC ? b->nCtas - 1 : b->nCtas));
                m = std::min<uint32_t>(m, k);
                const double tb = std::max(bigMax, sb / (m * ctaRate));
                const double ts = k < nC ? std::max(smallMax, ss / ((double)(b->nCtas - m) * warpsPerCta)) : 0.0;
                const double t = std::max(tb, ts);
                if (t < bestT) {
                    bestT = t;
                    bestK = k;
                    bestM = m;
                }
            }
        }
    std::vector<uint32_t> big(order.begin(), order.begin() + bestK), small(order.begin() + bestK, order.end());
    const uint32_t mCta = bestM;
    using Item = std::pair<double, uint32_t>;
    std::vector<std::vector<uint32_t>> ctaWhole(b->nCtas);
    {
        std::priority_queue<Item, std::vector<Item>, std::greater<Item>> q;
        for (uint32_t k = 0; k < mCta; ++k) q.push({0.0, k});
        for (uint32_t c : big) {
            Item it = q.top();
            q.pop();
            ctaWhole[it.second].push_back(c);
            q.push({it.first + cost[c] / ctaRate, it.second});
        }
    }
    std::priority_queue<Item, std::vector<Item>, std::greater<Item>> cta;
    for (uint32_t k = mCta; k < b->nCtas; ++k) cta.push({0.0, k});
    std::vector<std::vector<uint32_t>> ctaCells(b->nCtas);
    for (uint32_t c : small) {
        Item it = cta.top();
        cta.pop();
        ctaCells[it.second].push_back(c);
        // a CTA runs its warps concurrently: its load is spread over them
        cta.push({it.first + cost[c] / warpsPerCta, it.second});
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
    std::vector<uint32_t> cptr(b->nCtas + 1, 0), ccells;
    for (uint32_t k = 0; k < b->nCtas; ++k) {
        cptr[k + 1] = cptr[k] + (uint32_t)ctaWhole[k].size();
        ccells.insert(ccells.end(), ctaWhole[k].begin(), ctaWhole[k].end());
    }
    b->dWarpPtr = b->packBuf.up(ptr, b->st);
    b->dWarpCells = b->packBuf.up(cells, b->st);
    b->dCtaCellPtr = b->packBuf.up(cptr, b->st);
    b->dCtaCells = b->packBuf.up(ccells, b->st);
    b->nCtaWhole = mCta;
    if (b->packBuf.err == cudaSuccess) b->packBuf.err = cudaStreamSynchronize(b->st);
    if (b->packBuf.err != cudaSuccess) return cerr(b->packBuf.err, "batch packing");
    return HS_OK;
}

// ---- FP64 batch: drop-in layout per cell, shared tables ---------------------
// Mixed batch: the step at which an event of time t is delivered, the first
// step whose currTime = dt (step + 1) reaches t (SimpleSynHandler delivers
// the events with time <= currTime), as a 32-bit step count.
uint32_t deliveryStep(double t, double dt) {
    const double g = std::ceil(t / dt) - 3.0;
    uint64_t s = g > 0 ? (uint64_t)std::min(g, 4294967296.0) : 0;
    while (s < 0xffffffffull && !(t <= dt * (double)(s + 1))) ++s;
    return (uint32_t)std::min<uint64_t>(s, 0xffffffffu);
}

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
    b->synBase.assign(nC + 1, 0);
    for (uint32_t c = 0; c < nC; ++c) b->synBase[c + 1] = b->synBase[c] + b->plans[c].S;
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
    e = cudaMallocAsync(&b->arena.base, b->arena.size, b->st);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->arena.base, 0, b->arena.size, b->st);
    for (uint32_t c = 0; c < nC && e == cudaSuccess; ++c)
        e = layoutCell(b->plans[c], b->arena, b->dcs[c], b->spikeCap, b->st, &sh[c]);
    if (e != cudaSuccess) return cerr(e, "batch upload");
    b->dDcs = b->buf.alloc<DevCell>(nC);
    if (b->buf.err != cudaSuccess) return cerr(b->buf.err, "batch cells");
    b->evDesc.resize(nC);
    for (uint32_t c = 0; c < nC; ++c) b->evDesc[c] = {b->dcs[c].evPtr, b->dcs[c].evCur, b->dcs[c].evTime, b->dcs[c].evW};
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

// Star-form tree of one cell (hs_mixed.cuh): compartments 0..N-1 in the
// plan's Hines numbering, junction nodes N..T-1; children in CSR.
struct StarTree {
    uint32_t N = 0, T = 0, root = 0;
    std::vector<uint32_t> chPtr, ch;
    std::vector<double> diag, off;
};

int starTree(const CellPlan& P, StarTree& S) {
    const uint32_t N = P.N;
    std::vector<int64_t> mparent(N, -1);
    for (uint32_t i = 0; i < N; ++i)
        for (uint32_t c : P.children[i]) mparent[c] = i;
    int64_t root = -1;
    for (uint32_t i = 0; i < N; ++i)
        if (mparent[i] < 0) root = i;
    if (root < 0) return berr(HS_EINVAL, "mixed batch: no root compartment");
    std::vector<double> Ga(N), diag(N);
    for (uint32_t i = 0; i < N; ++i) {
        Ga[i] = 2.0 / P.Ra[i];
        diag[i] = P.Cm[i] / (P.dtSetup / 2.0) + 1.0 / P.Rm[i];
    }
    std::vector<std::vector<uint32_t>> tk(N);
    std::vector<double> toff(N, 0.0);
    for (uint32_t p = 0; p < N; ++p) {
        const std::vector<uint32_t>& chs = P.children[p];
        if (chs.size() == 1) {
            const uint32_t c = chs[0];
            const double g = Ga[p] * Ga[c] / (Ga[p] + Ga[c]);
            diag[p] += g;
            diag[c] += g;
            tk[p].push_back(c);
            toff[c] = -g;
        } else if (chs.size() >= 2) {
            const uint32_t J = (uint32_t)diag.size();
            double gsum = Ga[p];
            for (uint32_t c : chs) gsum += Ga[c];
            diag.push_back(gsum);
            toff.push_back(-Ga[p]);
            tk.push_back(std::vector<uint32_t>(chs.begin(), chs.end()));
            diag[p] += Ga[p];
            tk[p].push_back(J);
            for (uint32_t c : chs) {
                diag[c] += Ga[c];
                toff[c] = -Ga[c];
            }
        }
    }
    const uint32_t T = (uint32_t)diag.size();
    // every node reachable from the root exactly once
    std::vector<uint32_t> bfs;
    bfs.reserve(T);
    bfs.push_back((uint32_t)root);
    for (size_t k = 0; k < bfs.size() && bfs.size() <= T; ++k)
        for (uint32_t c : tk[bfs[k]]) bfs.push_back(c);
    if (bfs.size() != T) return berr(HS_EINVAL, "mixed batch: tree construction failed");
    for (uint32_t t = 0; t < T; ++t)
        if (tk[t].size() > 255) return berr(HS_ENOTSUP, "mixed batch: more than 255 children at a node");
    S.N = N;
    S.T = T;
    S.root = (uint32_t)root;
    S.chPtr.assign(T + 1, 0);
    for (uint32_t t = 0; t < T; ++t) S.chPtr[t + 1] = S.chPtr[t] + (uint32_t)tk[t].size();
    S.ch.reserve(S.chPtr[T]);
    for (uint32_t t = 0; t < T; ++t) S.ch.insert(S.ch.end(), tk[t].begin(), tk[t].end());
    S.diag = std::move(diag);
    S.off = std::move(toff);
    return HS_OK;
}

// Shared-memory bytes per forest node: D, R, OFF (8 B), TOPO (4 B), PAR (2 B);
// the kernel also keeps kSmemLevels level offsets and kWsLevels level
// counters (4 B each) there.
constexpr uint32_t kForestNodeBytes = 30;

// The rate tables of a mixed batch: one V table and one Ca table for all
// cells.  Every cell's table must lie on the same grid (min, max, rows, dx);
// their species (A/B column pairs, createLookupTables) are merged, a species
// with the same values in several cells stored once.  colMap[c][k] is the
// union column of column k of cell c's table (k even: the A of a species).
struct UnionTable {
    double min = 0, max = 0, dx = 0;
    uint32_t nPts = 0, nCol = 0;
    std::vector<double> data;                    // nPts x nCol
    std::vector<std::vector<int32_t>> colMap;    // per cell
};

int unionTables(HsBatch* b, bool ca, UnionTable& U) {
    const uint32_t nC = b->nCells;
    U = UnionTable();
    U.colMap.resize(nC);
    std::vector<std::vector<double>> species;    // column pairs of the union: A rows then B rows
    std::multimap<uint64_t, uint32_t> byHash;
    std::map<std::pair<uint64_t, size_t>, std::vector<int32_t>> byTable;   // distinct tables
    bool have = false;
    for (uint32_t c = 0; c < nC; ++c) {
        const Table& T = ca ? b->plans[c].caTable : b->plans[c].vTable;
        if (T.nCol == 0) continue;
        if (!have) {
            U.min = T.min, U.max = T.max, U.dx = T.dx, U.nPts = T.nPts;
            have = true;
        } else if (T.min != U.min || T.max != U.max || T.dx != U.dx || T.nPts != U.nPts) {
            return berr(HS_ENOTSUP, std::string("mixed batch: the cells' ") + (ca ? "Ca" : "V") +
                                        " rate tables lie on different grids (min, max, divisions)");
        }
        const auto key = std::make_pair(fnv(T.data.data(), T.data.size() * 8), T.data.size());
        auto it = byTable.find(key);
        if (it == byTable.end()) {
            std::vector<int32_t> map(T.nCol, -1);
            for (uint32_t s = 0; s + 1 < T.nCol; s += 2) {
                std::vector<double> col(2 * (size_t)T.nPts);
                for (uint32_t r = 0; r < T.nPts; ++r) {
                    col[r] = T.data[(size_t)r * T.nCol + s];
                    col[T.nPts + r] = T.data[(size_t)r * T.nCol + s + 1];
                }
                const uint64_t h = fnv(col.data(), col.size() * 8);
                int32_t u = -1;
                for (auto r = byHash.equal_range(h); r.first != r.second; ++r.first)
                    if (species[r.first->second] == col) u = (int32_t)r.first->second;
                if (u < 0) {
                    u = (int32_t)species.size();
                    species.push_back(std::move(col));
                    byHash.emplace(h, (uint32_t)u);
                }
                map[s] = 2 * u;
                map[s + 1] = 2 * u + 1;
            }
            it = byTable.emplace(key, std::move(map)).first;
        }
        U.colMap[c] = it->second;
    }
    U.nCol = 2 * (uint32_t)species.size();
    U.data.assign((size_t)U.nPts * U.nCol, 0.0);
    for (size_t u = 0; u < species.size(); ++u)
        for (uint32_t r = 0; r < U.nPts; ++r) {
            U.data[(size_t)r * U.nCol + 2 * u] = species[u][r];
            U.data[(size_t)r * U.nCol + 2 * u + 1] = species[u][U.nPts + r];
        }
    return HS_OK;
}

int buildMixed(HsBatch* b) {
    const uint32_t nC = b->nCells;
    for (const CellPlan& P : b->plans)
        if (P.nDif)
            return berr(HS_ENOTSUP, "mixed batch: tick-1 external calcium objects (DifShell, DifBuffer, MMPump) "
                                    "are stepped by the FP64 solvers only");
    MixHost& H = b->mh;
    H = MixHost();
    // one V table and one Ca table for the batch: the union of the cells'
    UnionTable V0, C0;
    int urc = unionTables(b, false, V0);
    if (urc == HS_OK) urc = unionTables(b, true, C0);
    if (urc != HS_OK) return urc;
    // forest capacity from the shared memory of a CTA
    int optin = 0, perSm = 0;
    cudaError_t ce = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, b->device);
    if (ce == cudaSuccess) ce = cudaDeviceGetAttribute(&perSm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, b->device);
    if (ce != cudaSuccess) return cerr(ce, "shared memory size");
    const uint32_t perCta =
        std::min<uint32_t>((uint32_t)optin, (uint32_t)perSm / std::max<uint32_t>(1, b->ctasPerSm) - 1024) / 256 * 256;
    const uint32_t reserve = (kSmemLevels + kWsLevels) * 4;
    if (perCta < reserve + 8 * kForestNodeBytes) return berr(HS_EINVAL, "too many CTAs per SM");
    uint32_t cap = std::min<uint32_t>(kMaxForestNodes, (perCta - reserve) / kForestNodeBytes) / 8 * 8;
    // a cluster keeps only D and R (16 B a node) of its forest in rank 0's
    // shared memory, after the level offsets, counters and barrier word
    const uint32_t reserveCl = (kSmemLevels + kWsLevels + 4) * 4;
    if (b->clusterCtas > 1) cap = std::min<uint32_t>(kMaxForestNodes, (perCta - reserveCl) / 16) / 8 * 8;
    if (b->forestNodes) cap = std::min(cap, b->forestNodes / 8 * 8);
    if (cap < 8) return berr(HS_EINVAL, "forest_nodes too small");
    b->mixCap = cap;
    b->mixSmem = (reserve + cap * kForestNodeBytes + 15) / 16 * 16;
    if (b->clusterCtas > 1) {
        b->mixSmem = reserveCl + 16 * cap;
        b->mixStageCap = (b->mixSmem - reserveCl) / kForestNodeBytes / 8 * 8;
        if (b->threadsPerCta <= 32 * (b->elimWarps ? b->elimWarps : 4))
            return berr(HS_EINVAL, "cluster_ctas: threads_per_cta must exceed the eliminator warps");
    }

    // 1. star trees
    std::vector<StarTree> trees(nC);
    for (uint32_t c = 0; c < nC; ++c) {
        int rc = starTree(b->plans[c], trees[c]);
        if (rc != HS_OK) return rc;
        if (trees[c].T > kMaxForestNodes) return berr(HS_ENOTSUP, "mixed batch: a cell has more than 65535 nodes");
    }
    // 2. packing: cells to the CTAs of one wave by node count (longest
    // processing time first), then within a CTA into forests: cells that fit
    // the shared-memory capacity first-fit decreasing into shared forests,
    // larger cells into global forests of up to 65535 nodes
    uint32_t nCtas = std::max<uint32_t>(1, b->nSm * b->ctasPerSm);
    if (b->maxCtas) nCtas = std::min(nCtas, b->maxCtas);
    // with clusters, a "CTA" of the packing below is a group of clusterCtas
    // CTAs, and every forest goes to global memory
    const bool clustered = b->clusterCtas > 1;
    if (clustered) nCtas = std::max<uint32_t>(1, nCtas / b->clusterCtas);
    std::vector<uint32_t> order(nC);
    for (uint32_t c = 0; c < nC; ++c) order[c] = c;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) { return trees[x].T > trees[y].T; });
    using Item = std::pair<double, uint32_t>;
    std::priority_queue<Item, std::vector<Item>, std::greater<Item>> pq;
    for (uint32_t k = 0; k < nCtas; ++k) pq.push({0.0, k});
    std::vector<std::vector<uint32_t>> ctaCells(nCtas);
    for (uint32_t c : order) {
        Item it = pq.top();
        pq.pop();
        ctaCells[it.second].push_back(c);
        pq.push({it.first + trees[c].T * (trees[c].T > cap ? 1.5 : 1.0), it.second});
    }
    struct ForestPlan {
        std::vector<uint32_t> cells;
        uint32_t nodes = 0;
        bool shared = true;
    };
    std::vector<ForestPlan> forests;
    std::vector<uint32_t> ctaPtr(nCtas + 1, 0), ctaForests;
    for (uint32_t k = 0; k < nCtas; ++k) {
        std::vector<ForestPlan> fs;
        for (uint32_t c : ctaCells[k]) {      // decreasing size
            const uint32_t T = trees[c].T;
            const bool sh = T <= cap;
            if (clustered && !sh)
                return berr(HS_ENOTSUP, "mixed batch: a cell too large for a cluster's shared-memory forest");
            const uint32_t lim = sh ? cap : kMaxForestNodes;
            size_t f = 0;
            while (f < fs.size() && (fs[f].shared != sh || fs[f].nodes + T > lim)) ++f;
            if (f == fs.size()) {
                fs.emplace_back();
                fs.back().shared = sh;
            }
            fs[f].cells.push_back(c);
            fs[f].nodes += T;
        }
        for (ForestPlan& f : fs) {
            ctaForests.push_back((uint32_t)forests.size());
            forests.push_back(std::move(f));
        }
        ctaPtr[k + 1] = (uint32_t)ctaForests.size();
    }
    // launch only CTAs that hold forests (a small batch leaves the other SMs
    // to concurrent batches)
    {
        std::vector<uint32_t> kept(1, 0);
        for (uint32_t k = 0; k < nCtas; ++k)
            if (ctaPtr[k + 1] > ctaPtr[k]) kept.push_back(ctaPtr[k + 1]);
        ctaPtr.swap(kept);
    }
    const uint32_t busy = (uint32_t)ctaPtr.size() - 1;
    // 3. node numbering: forest after forest, level-major inside a forest
    std::vector<std::vector<uint32_t>> posOf(nC);
    std::vector<std::pair<uint32_t, uint32_t>> nodeCT;    // (cell, tree node) of each global node
    std::vector<uint8_t> nodeLevel;                       // forest level, capped at 255
    std::vector<MixForest> fdev(forests.size());
    std::vector<uint32_t> levelPtr, forestCells;
    for (size_t fi = 0; fi < forests.size(); ++fi) {
        const ForestPlan& FP = forests[fi];
        MixForest& F = fdev[fi];
        std::memset(&F, 0, sizeof(F));
        F.node0 = (uint32_t)nodeCT.size();
        F.nNodes = FP.nodes;
        F.level0 = (uint32_t)levelPtr.size();
        F.cell0 = (uint32_t)forestCells.size();
        F.nCells = (uint32_t)FP.cells.size();
        F.shared = FP.shared ? 1 : 0;
        forestCells.insert(forestCells.end(), FP.cells.begin(), FP.cells.end());
        std::vector<std::pair<uint32_t, uint32_t>> cur, next;
        for (uint32_t c : FP.cells) {
            cur.push_back({c, trees[c].root});
            posOf[c].assign(trees[c].T, 0);
        }
        levelPtr.push_back(0);
        while (!cur.empty()) {
            const uint8_t lv = (uint8_t)std::min<size_t>(255, levelPtr.size() - F.level0 - 1);
            for (auto& ct : cur) {
                posOf[ct.first][ct.second] = (uint32_t)nodeCT.size();
                nodeCT.push_back(ct);
                nodeLevel.push_back(lv);
            }
            levelPtr.push_back((uint32_t)(nodeCT.size() - F.node0));
            next.clear();
            for (auto& ct : cur) {
                const StarTree& S = trees[ct.first];
                for (uint32_t k = S.chPtr[ct.second]; k < S.chPtr[ct.second + 1]; ++k) next.push_back({ct.first, S.ch[k]});
            }
            // junction nodes after compartments; a node's children keep
            // their order and stay contiguous (they are all of one kind)
            std::stable_partition(next.begin(), next.end(),
                                  [&](const std::pair<uint32_t, uint32_t>& ct) { return ct.second < trees[ct.first].N; });
            cur.swap(next);
        }
        F.nLevels = (uint32_t)(levelPtr.size() - F.level0 - 1);
        if (nodeCT.size() - F.node0 != F.nNodes) return berr(HS_EINVAL, "mixed batch: forest layout failed");
        if (clustered && F.nLevels > kWsLevels - 1)
            return berr(HS_ENOTSUP, "mixed batch: a forest stepped by a cluster has more than 255 tree levels");
    }
    const uint32_t nN = (uint32_t)nodeCT.size();
    // 4. per-cell lists: inject entries, stimulus, SpikeGens; model maps
    H.cells.resize(nC);
    H.nodeOf.resize(nC);
    H.chanSlot.resize(nC);
    H.c2dNode.resize(nC);
    H.synGlobal.resize(nC);
    H.poolOf.resize(nC);
    b->injEntryOf.clear();
    std::vector<double> injVal, stimValue;
    std::vector<uint32_t> stimStep, stimEntry, sgNode;
    std::vector<float> sgThresh, sgRefract;
    std::vector<int32_t> sgEdge;
    std::vector<std::vector<int32_t>> injAt(nC), c2dAt(nC);
    std::vector<std::vector<uint32_t>> synPtr(nC), synIdx(nC);
    for (uint32_t ci = 0; ci < nC; ++ci) {
        const CellPlan& P = b->plans[ci];
        const uint32_t N = P.N;
        MixCellRange& R = H.cells[ci];
        std::memset(&R, 0, sizeof(R));
        H.nodeOf[ci].assign(P.hinesOf.size(), -1);
        H.chanSlot[ci].assign(P.chanSolverOf.size(), -1);
        H.c2dNode[ci].assign(P.K2, -1);
        H.synGlobal[ci].assign(P.S, -1);
        for (size_t m = 0; m < P.hinesOf.size(); ++m)
            if (P.hinesOf[m] >= 0) H.nodeOf[ci][m] = posOf[ci][P.hinesOf[m]];
        H.poolOf[ci].assign(P.poolSolverOf.size(), -1);
        injAt[ci].assign(N, -1);
        R.inj0 = (uint32_t)injVal.size();
        for (uint32_t i = 0; i < N; ++i)
            if (P.injPresent[i]) {
                injAt[ci][i] = (int32_t)(injVal.size() - R.inj0);
                injVal.push_back(P.injBasal[i]);
            }
        for (uint32_t k = 0; k < P.stimCompt.size(); ++k)
            if (injAt[ci][P.stimCompt[k]] < 0) {
                injAt[ci][P.stimCompt[k]] = (int32_t)(injVal.size() - R.inj0);
                injVal.push_back(0.0);
            }
        R.nInj = (uint32_t)injVal.size() - R.inj0;
        b->injEntryOf.emplace_back(P.hinesOf.size(), -1);
        for (uint32_t i = 0; i < N; ++i)
            if (injAt[ci][i] >= 0) b->injEntryOf.back()[P.modelOf[i]] = (int32_t)R.inj0 + injAt[ci][i];
        R.stim0 = (uint32_t)stimStep.size();
        for (uint32_t k = 0; k < P.stimCompt.size(); ++k) {
            stimStep.push_back(P.stimStep[k]);
            stimEntry.push_back((uint32_t)injAt[ci][P.stimCompt[k]]);
            stimValue.push_back(P.stimValue[k]);
        }
        R.nStim = (uint32_t)stimStep.size() - R.stim0;
        R.sg0 = (uint32_t)sgNode.size();
        for (uint32_t k = 0; k < P.SG; ++k) {
            sgNode.push_back(posOf[ci][P.sgCompt[k]]);
            sgThresh.push_back((float)P.sgThreshold[k]);
            sgRefract.push_back((float)P.sgRefract[k]);
            sgEdge.push_back(P.sgEdge[k]);
        }
        R.nSg = P.SG;
        c2dAt[ci].assign(N, -1);
        for (uint32_t k = 0; k < P.K2; ++k) {
            if (c2dAt[ci][P.c2dCompt[k]] >= 0)
                return berr(HS_ENOTSUP, "mixed batch: more than one HHChannel2D in a compartment");
            c2dAt[ci][P.c2dCompt[k]] = (int32_t)k;
        }
        synPtr[ci].assign(N + 1, 0);
        for (uint32_t k = 0; k < P.S; ++k) synPtr[ci][P.synCompt[k] + 1]++;
        for (uint32_t i = 0; i < N; ++i) synPtr[ci][i + 1] += synPtr[ci][i];
        synIdx[ci].assign(P.S, 0);
        std::vector<uint32_t> fill(synPtr[ci].begin(), synPtr[ci].end() - 1);
        for (uint32_t k = 0; k < P.S; ++k) synIdx[ci][fill[P.synCompt[k]]++] = k;   // creation order per compartment
    }
    // 5. per-node arrays in global node order
    std::vector<float> vtab(V0.data.begin(), V0.data.end()), catab(C0.data.begin(), C0.data.end());
    std::map<std::tuple<const double*, const double*, uint32_t, uint32_t>, int> g2dIndex;
    std::vector<float> g2d, g2dGeom;
    std::vector<uint64_t> g2dOff;
    std::vector<uint32_t> g2dN;
    struct ChanKey {          // a channel type with its general powers (for dedup)
        ChanType t;
        ChanPow p;
    };
    std::vector<ChanKey> ctypes;
    std::vector<C2dType> ktypes;
    const uint64_t ld = (nN + 31) / 32 * 32;
    std::vector<uint32_t> nodeInfo(nN), ctype4(nN), topo(nN), injIdx(nN, 0), syn0;
    std::vector<uint16_t> par(nN, (uint16_t)kNoParent);
    std::vector<double> off(nN), HS2(nN), CmByDt(nN), EmByRm(nN);
    std::vector<float> gbarS((size_t)kMaxChan * ld, 0.f);
    std::vector<float2> stateS((size_t)3 * kMaxChan * ld, make_float2(0.f, 0.f));
    auto pair = [](double x) {
        const float hi = (float)x;
        return make_float2(hi, (float)(x - (double)hi));
    };
    std::vector<float> poolBasal(nN, 0.f), poolG1(nN, 0.f), poolF2(nN, 0.f), poolCeil(nN, 0.f), poolFloor(nN, 0.f);
    std::vector<float> k2gbar(nN, 0.f), k2x0(nN, 0.f);
    std::vector<uint8_t> synTypeV;
    H.initVm.assign(nN, 0.0);
    syn0.reserve(nN + 1);
    for (size_t fi = 0; fi < forests.size(); ++fi) {
        const MixForest& F = fdev[fi];
        for (uint32_t g = F.node0; g < F.node0 + F.nNodes; ++g) {
            const uint32_t ci = nodeCT[g].first, t = nodeCT[g].second;
            const CellPlan& P = b->plans[ci];
            const StarTree& S = trees[ci];
            const bool center = t >= S.N;
            const uint32_t nch = S.chPtr[t + 1] - S.chPtr[t];
            topo[g] = (nch ? posOf[ci][S.ch[S.chPtr[t]]] - F.node0 : 0) | (nch << 16) | ((uint32_t)nodeLevel[g] << 24);
            for (uint32_t k = S.chPtr[t]; k < S.chPtr[t + 1]; ++k) par[posOf[ci][S.ch[k]]] = (uint16_t)(g - F.node0);
            off[g] = S.off[t];
            HS2[g] = S.diag[t];
            uint32_t info = (center ? kNodeCenter : 0) | ((uint32_t)kNoType << 8);
            uint32_t types = 0xFFFFFFFFu;
            syn0.push_back((uint32_t)synTypeV.size());
            if (!center) {
                CmByDt[g] = P.CmByDt[t];
                EmByRm[g] = P.EmByRm[t];
                H.initVm[g] = P.initVm[t];
                if (injAt[ci][t] >= 0) {
                    info |= kNodeInject;
                    injIdx[g] = H.cells[ci].inj0 + (uint32_t)injAt[ci][t];
                }
                const uint32_t pb0 = P.poolPtr[t], pe0 = P.poolPtr[t + 1];
                if (pe0 - pb0 > 1) return berr(HS_ENOTSUP, "mixed batch: more than one Ca pool in a compartment");
                if (pe0 > pb0) {
                    info |= kNodePool;
                    H.poolOf[ci][P.poolModel[pb0]] = g;
                    poolBasal[g] = (float)P.CaBasal[pb0];
                    poolG1[g] = (float)(1.0 - P.f1[pb0]);     // decay per step, from FP64
                    poolF2[g] = (float)P.f2[pb0];
                    poolCeil[g] = (float)P.ceiling[pb0];
                    poolFloor[g] = (float)P.floor_[pb0];
                }
                const uint32_t q0 = P.chanPtr[t], q1 = P.chanPtr[t + 1];
                if (q1 - q0 > (uint32_t)kMaxChan)
                    return berr(HS_ENOTSUP, "mixed batch: more than 4 HHChannels in a compartment");
                for (uint32_t q = q0; q < q1; ++q) {
                    ChanKey key;
                    std::memset(&key, 0, sizeof(key));
                    ChanType& ty = key.t;
                    ty.ek = (float)P.Ek[q];
                    ty.xp = powCode(P.Xpow[q], key.p.x);
                    ty.yp = powCode(P.Ypow[q], key.p.y);
                    ty.zp = powCode(P.Zpow[q], key.p.z);
                    ty.instant = (int8_t)P.instant[q];
                    // columns of the union tables; a Z gate on its pool reads the
                    // Ca table, any other gate the V table (with the column
                    // number it has, as HSolveActive::advanceChannels does)
                    const bool zCaTab = P.Zpow[q] > 0.0 && P.zSrc[q] >= 0;
                    const std::vector<int32_t>& vm = V0.colMap[ci];
                    const std::vector<int32_t>& cm = C0.colMap[ci];
                    auto col = [](const std::vector<int32_t>& m, int32_t k) -> int32_t {
                        return k < 0 ? 0 : (size_t)k < m.size() ? m[k] : -1;
                    };
                    const int32_t cx = col(vm, P.colX[q]), cy = col(vm, P.colY[q]);
                    const int32_t cz = col(zCaTab ? cm : vm, P.colZ[q]);
                    if (cx < 0 || cy < 0 || cz < 0 || cx > 0x7FFF || cy > 0x7FFF || cz > 0x7FFF)
                        return berr(HS_ENOTSUP, "mixed batch: a gate column outside its rate table");
                    ty.colX = (int16_t)cx;
                    ty.colY = (int16_t)cy;
                    ty.colZ = (int16_t)cz;
                    if (zCaTab) {
                        if (P.zSrc[q] != (int32_t)pb0 || pe0 == pb0)
                            return berr(HS_ENOTSUP, "mixed batch: Ca-dependent gate reads another compartment's pool");
                        ty.zCa = 1;
                    }
                    if (P.caTarget[q] >= 0) {
                        if (P.caTarget[q] != (int32_t)pb0 || pe0 == pb0)
                            return berr(HS_ENOTSUP, "mixed batch: channel feeds another compartment's pool");
                        ty.caTarget = 1;
                    }
                    const int ti = typeIndex(ctypes, key, kMaxChanTypes - 1);
                    if (ti < 0) return berr(HS_ENOTSUP, "mixed batch: too many channel types");
                    const uint32_t j = q - q0;
                    types = (types & ~(0xFFu << (8 * j))) | ((uint32_t)ti << (8 * j));
                    gbarS[(size_t)j * ld + g] = (float)(P.Gbar[q] * P.modulation[q]);
                    H.chanSlot[ci][P.chanModel[q]] = (int64_t)g * kMaxChan + j;
                    int s = P.stateOff[q];
                    if (P.Xpow[q] > 0.0) stateS[(size_t)(3 * j) * ld + g] = pair(P.state0[s++]);
                    if (P.Ypow[q] > 0.0) stateS[(size_t)(3 * j + 1) * ld + g] = pair(P.state0[s++]);
                    if (P.Zpow[q] > 0.0) stateS[(size_t)(3 * j + 2) * ld + g] = pair(P.state0[s++]);
                    if (P.Xpow[q] > 0.0) info |= 1u << (kNodeGateShift + 3 * j);
                    if (P.Ypow[q] > 0.0) info |= 1u << (kNodeGateShift + 3 * j + 1);
                    if (P.Zpow[q] > 0.0) info |= 1u << (kNodeGateShift + 3 * j + 2);
                }
                const int32_t kk = c2dAt[ci][t];
                if (kk >= 0) {
                    const Gate2D& G = P.gates2d[P.c2dGate[kk]];
                    auto key = std::make_tuple(G.srcA, G.srcB, G.nx, G.ny);
                    auto it = g2dIndex.find(key);
                    if (it == g2dIndex.end()) {
                        if (g2dIndex.size() >= 127) return berr(HS_ENOTSUP, "mixed batch: too many 2-D tables");
                        const int gi = (int)g2dN.size() / 2;
                        const size_t nn = (size_t)G.nx * G.ny;
                        g2dOff.push_back(g2d.size());
                        const size_t o = g2d.size();
                        g2d.resize(o + 2 * nn);
                        for (size_t i = 0; i < nn; ++i) {
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
                    ky.ek = (float)P.c2dEk[kk];
                    ky.xp = powCode(P.c2dXpow[kk], ky.xpf);
                    if (P.c2dConc2[kk] >= 0 || P.c2dDep0[kk] == 2 || P.c2dDep1[kk] == 2)
                        return berr(HS_ENOTSUP, "mixed batch: HHChannel2D on a second concentration");
                    if (P.c2dConc1[kk] >= 0 && (P.c2dConc1[kk] != (int32_t)pb0 || pe0 == pb0))
                        return berr(HS_ENOTSUP, "mixed batch: HHChannel2D reads another compartment's pool");
                    auto dep = [](int32_t d) -> int8_t { return d < 0 ? -1 : d == 0 ? 0 : d == 1 ? 1 : -2; };
                    ky.dep0 = dep(P.c2dDep0[kk]);
                    ky.dep1 = dep(P.c2dDep1[kk]);
                    ky.instant = (int8_t)P.c2dInstant[kk];
                    ky.gate = (int8_t)it->second;
                    const int ti = typeIndex(ktypes, ky, kMaxC2dTypes - 1);
                    if (ti < 0) return berr(HS_ENOTSUP, "mixed batch: too many HHChannel2D types");
                    info = (info & ~(0xFFu << 8)) | ((uint32_t)ti << 8);
                    k2gbar[g] = (float)(P.c2dGbar[kk] * P.c2dMod[kk]);
                    H.c2dNode[ci][kk] = g;
                    k2x0[g] = (float)P.c2dX0[kk];
                }
                if (synPtr[ci][t + 1] > synPtr[ci][t]) info |= kNodeSyn;
                for (uint32_t q = synPtr[ci][t]; q < synPtr[ci][t + 1]; ++q) {
                    const uint32_t kk2 = synIdx[ci][q];
                    auto key = std::make_tuple(P.synTau1[kk2], P.synTau2[kk2], P.synEk[kk2]);
                    size_t ti = 0;
                    while (ti < H.synTypeKey.size() && H.synTypeKey[ti] != key) ++ti;
                    if (ti == H.synTypeKey.size()) {
                        if (ti >= (size_t)kMaxSynTypes) return berr(HS_ENOTSUP, "mixed batch: too many SynChan types");
                        H.synTypeKey.push_back(key);
                    }
                    synTypeV.push_back((uint8_t)ti);
                    H.synGlobal[ci][kk2] = (int64_t)H.synGbar.size();
                    H.synGbar.push_back(P.synGbar[kk2]);
                    H.synTau1.push_back(P.synTau1[kk2]);
                    H.synTau2.push_back(P.synTau2[kk2]);
                    H.synMod.push_back(P.synMod[kk2]);
                    H.evStart.push_back((uint32_t)H.evTime.size());
                    for (uint32_t e = P.evPtr[kk2]; e < P.evPtr[kk2 + 1]; ++e) {
                        H.evTime.push_back(P.evTime[e]);
                        H.evW.push_back(P.evW[e]);
                    }
                    H.evEnd.push_back((uint32_t)H.evTime.size());
                }
            }
            nodeInfo[g] = info;
            ctype4[g] = types;
        }
    }
    syn0.push_back((uint32_t)synTypeV.size());
    H.nNodes = nN;
    H.c2dX0 = k2x0;
    H.nForests = (uint32_t)forests.size();
    H.nShared = 0;
    for (const ForestPlan& f : forests) H.nShared += f.shared ? 1 : 0;
    trees.clear();
    // 6. upload
    DevBuf& D = b->buf;
    cudaStream_t st = b->st;
    MixBatch& m = b->mb;
    std::memset(&m, 0, sizeof(m));
    m.nCells = nC;
    m.nForests = (uint32_t)fdev.size();
    m.ld = ld;
    m.cells = D.up(H.cells, st);
    m.forests = D.up(fdev, st);
    m.forestStep = D.zeros<unsigned long long>(fdev.size(), st);
    m.err = D.zeros<uint32_t>(1, st);
    {
        std::vector<uint32_t> cellOf(nN);
        for (uint32_t g = 0; g < nN; ++g) cellOf[g] = nodeCT[g].first;
        m.cellOf = D.up(cellOf, st);
        b->dStopStep = D.up(std::vector<unsigned long long>(nC, ~0ull), st);
        m.stopStep = b->dStopStep;
        b->dForestStop = D.up(std::vector<unsigned long long>(fdev.size(), ~0ull), st);
        m.forestStop = b->dForestStop;
        b->forestCellPtr.assign(fdev.size() + 1, 0);
        for (size_t fi = 0; fi < fdev.size(); ++fi) b->forestCellPtr[fi + 1] = fdev[fi].cell0 + fdev[fi].nCells;
        b->forestCellIdx = forestCells;
    }
    m.forestCells = D.up(forestCells, st);
    m.levelPtr = D.up(levelPtr, st);
    m.nodeInfo = D.up(nodeInfo, st);
    m.ctype4 = D.up(ctype4, st);
    m.topo = D.up(topo, st);
    m.par = D.up(par, st);
    m.injIdx = D.up(injIdx, st);
    m.off = D.up(off, st);
    m.HS2 = D.up(HS2, st);
    m.CmByDt = D.up(CmByDt, st);
    m.EmByRm = D.up(EmByRm, st);
    m.V = D.up(H.initVm, st);
    if (H.nShared < H.nForests) {
        m.elimD = D.zeros<double>(nN, st);
        m.elimR = D.zeros<double>(nN, st);
    }
    m.caG = D.zeros<float>(nN, st);
    m.caGE = D.zeros<float>(nN, st);
    m.gbar = D.up(gbarS, st);
    m.state = D.up(stateS, st);
    m.poolC = D.zeros<float>(nN, st);
    m.poolCa = D.up(poolBasal, st);
    m.poolG1 = D.up(poolG1, st);
    m.poolF2 = D.up(poolF2, st);
    m.poolBasal = D.up(poolBasal, st);
    m.poolCeil = D.up(poolCeil, st);
    m.poolFloor = D.up(poolFloor, st);
    m.k2gbar = D.up(k2gbar, st);
    m.k2x = D.up(k2x0, st);
    m.g2d = D.up(g2d, st);
    m.g2dOff = D.up(g2dOff, st);
    m.g2dGeom = D.up(g2dGeom, st);
    m.g2dN = D.up(g2dN, st);
    m.syn0 = D.up(syn0, st);
    m.synType = D.up(synTypeV, st);
    m.synX = D.zeros<float>(synTypeV.size(), st);
    m.synY = D.zeros<float>(synTypeV.size(), st);
    m.synGk = D.zeros<float2>(synTypeV.size(), st);
    {
        std::vector<uint32_t> synCell(synTypeV.size());
        for (uint32_t g = 0; g < nN; ++g)
            for (uint32_t k = syn0[g]; k < syn0[g + 1]; ++k) synCell[k] = nodeCT[g].first;
        m.synCell = D.up(synCell, st);
    }
    m.evCur = D.up(H.evStart, st);
    m.evEnd = D.up(H.evEnd, st);
    b->dEvCurDesc = m.evCur;
    b->dEvEndDesc = m.evEnd;
    b->dEvStep = D.zeros<uint32_t>(H.evTime.size(), st);
    b->dEvAct = D.zeros<float>(H.evTime.size(), st);
    b->dSynNorm = D.zeros<float>(synTypeV.size(), st);
    m.evStep = b->dEvStep;
    m.evAct = b->dEvAct;
    m.synNorm = b->dSynNorm;
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
    // per-node arrays the assembly reads, for the L2 prefetch
    {
        uint32_t gateUse = 0, slotUse = 0, anyPool = 0, anyK2 = 0, anySyn = 0;
        for (uint32_t g = 0; g < nN; ++g) {
            gateUse |= nodeInfo[g] >> kNodeGateShift;
            for (int j = 0; j < kMaxChan; ++j)
                if (((ctype4[g] >> (8 * j)) & 0xFF) != kNoType) slotUse |= 1u << j;
            anyPool |= nodeInfo[g] & kNodePool;
            anyK2 |= ((nodeInfo[g] >> 8) & 0xFF) != kNoType;
            anySyn |= nodeInfo[g] & kNodeSyn;
        }
        auto add = [&](const void* p, uint32_t elem, uint64_t n) {
            if (m.nPf < (uint32_t)kMaxPrefetch) m.pf[m.nPf++] = PrefetchArr{p, elem, (uint32_t)n};
        };
        add(m.nodeInfo, 4, nN);
        add(m.ctype4, 4, nN);
        add(m.V, 8, nN);
        add(m.HS2, 8, nN);
        add(m.CmByDt, 8, nN);
        add(m.EmByRm, 8, nN);
        for (int k = 0; k < 3 * kMaxChan; ++k)
            if ((gateUse >> k) & 1u) add(m.state + (size_t)k * ld, 8, ld);
        for (int j = 0; j < kMaxChan; ++j)
            if ((slotUse >> j) & 1u) add(m.gbar + (size_t)j * ld, 4, ld);
        if (anyPool) {
            add(m.poolC, 4, nN);
            add(m.poolCa, 4, nN);
            add(m.poolG1, 4, nN);
            add(m.poolF2, 4, nN);
            add(m.poolBasal, 4, nN);
            add(m.caG, 4, nN);
            add(m.caGE, 4, nN);
        }
        if (anyK2) {
            add(m.k2x, 4, nN);
            add(m.k2gbar, 4, nN);
        }
        if (anySyn) add(m.syn0, 4, nN + 1);
    }
    b->dCtaPtr = D.up(ctaPtr, st);
    b->dCtaForests = D.up(ctaForests, st);
    b->nCtas = busy;
    if (D.err != cudaSuccess) return cerr(D.err, "mixed batch upload");
    std::vector<ChanType> ctT;
    std::vector<ChanPow> ctP;
    for (const ChanKey& k : ctypes) {
        ctT.push_back(k.t);
        ctP.push_back(k.p);
    }
    m.chanTypes = D.up(ctT, st);
    m.chanPow = D.up(ctP, st);
    m.c2dTypes = D.up(ktypes, st);
    b->dSynTypes = D.zeros<SynType>(kMaxSynTypes, st);
    m.synTypes = b->dSynTypes;
    if (D.err != cudaSuccess) return cerr(D.err, "mixed batch types");
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cerr(e, "mixed batch types");
    return HS_OK;
}

// ---- run-time synaptic events ----------------------------------------------------
// Back to the description's queues (reinit, re-layout): SimpleSynHandler's
// vReinit empties its queue.  The owned queue is freed in stream order.
void dropRuntimeEvents(HsBatch* b) {
    b->pendSyn.clear();
    b->pendTime.clear();
    b->pendW.clear();
    if (!b->evOwned) return;
    if (b->precision == HS_PREC_FP64) {
        for (uint32_t c = 0; c < b->nCells; ++c) {
            b->dcs[c].evPtr = b->evDesc[c].ptr;
            b->dcs[c].evCur = b->evDesc[c].cur;
            b->dcs[c].evTime = b->evDesc[c].time;
            b->dcs[c].evW = b->evDesc[c].w;
        }
    } else {
        b->mb.evCur = b->dEvCurDesc;
        b->mb.evEnd = b->dEvEndDesc;
        b->mb.evStep = b->dEvStep;
        b->mb.evAct = b->dEvAct;
    }
    b->evBuf.freeAll();
    b->evBuf.err = cudaSuccess;
    b->evHostPtr.clear();
    b->evHostTime.clear();
    b->evHostW.clear();
    b->dEvOwnCur = nullptr;
    b->evOwned = false;
}

// Hands the pushed events to the device before a process call.  The queue
// over every SynChan of the batch is rebuilt on the host from the device
// cursors (mergeEventQueue, hs_events.h: undelivered events merged with the
// pushes in time order) and uploaded to a new owned buffer; the kernels walk
// it exactly as they walk the description's events.  The old queue stays in
// place until the new one is on the device.
int flushRuntimeEvents(HsBatch* b) {
    if (b->pendSyn.empty()) return HS_OK;
    const bool fp64 = b->precision == HS_PREC_FP64;
    MixHost& H = b->mh;
    const uint32_t S = fp64 ? b->synBase.back() : (uint32_t)H.synGbar.size();
    cudaError_t e = cudaStreamSynchronize(b->st);
    if (e != cudaSuccess) return cerr(e, "push events");
    std::vector<uint32_t> cur(S), descPtr;
    std::vector<double> descTime, descW;
    std::vector<uint32_t> cellEv0;            // FP64 description: first event of each cell
    if (!b->evOwned && fp64) {
        descPtr.resize((size_t)S + 1);
        cellEv0.resize(b->nCells);
        for (uint32_t c = 0; c < b->nCells; ++c) {
            const CellPlan& P = b->plans[c];
            const uint32_t off = (uint32_t)descTime.size();
            cellEv0[c] = off;
            for (uint32_t j = 0; j < P.S; ++j) descPtr[b->synBase[c] + j] = off + P.evPtr[j];
            descTime.insert(descTime.end(), P.evTime.begin(), P.evTime.end());
            descW.insert(descW.end(), P.evW.begin(), P.evW.end());
            if (P.S && e == cudaSuccess)
                e = cudaMemcpyAsync(cur.data() + b->synBase[c], b->evDesc[c].cur, P.S * sizeof(uint32_t),
                                    cudaMemcpyDeviceToHost, b->st);
        }
        descPtr[S] = (uint32_t)descTime.size();
    } else if (!b->evOwned) {
        descPtr = H.evStart;
        descPtr.push_back(S ? H.evEnd.back() : 0u);
        if (S) e = cudaMemcpyAsync(cur.data(), b->mb.evCur, S * sizeof(uint32_t), cudaMemcpyDeviceToHost, b->st);
    } else if (S) {
        e = cudaMemcpyAsync(cur.data(), b->dEvOwnCur, S * sizeof(uint32_t), cudaMemcpyDeviceToHost, b->st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
    if (e != cudaSuccess) return cerr(e, "push events");
    if (!b->evOwned && fp64)
        for (uint32_t c = 0; c < b->nCells; ++c)
            for (uint32_t j = 0; j < b->plans[c].S; ++j) cur[b->synBase[c] + j] += cellEv0[c];
    const std::vector<uint32_t>& ptr = b->evOwned ? b->evHostPtr : descPtr;
    const std::vector<double>& tm = b->evOwned ? b->evHostTime : (fp64 ? descTime : H.evTime);
    const std::vector<double>& wt = b->evOwned ? b->evHostW : (fp64 ? descW : H.evW);
    std::vector<uint32_t> nptr;
    std::vector<double> nt, nw;
    if (!mergeEventQueue(S, ptr, tm, wt, cur, b->pendSyn, b->pendTime, b->pendW, nptr, nt, nw))
        return berr(HS_ENOMEM, "too many queued synaptic events");
    DevBuf nb;
    nb.st = b->st;
    const size_t m = nt.size();
    if (fp64) {
        uint32_t* idx = nb.up(nptr, b->st);
        std::vector<double> tw(nt);
        tw.insert(tw.end(), nw.begin(), nw.end());
        double* ev = nb.up(tw, b->st);
        if (nb.err == cudaSuccess) nb.err = cudaStreamSynchronize(b->st);
        if (nb.err != cudaSuccess) {
            cudaError_t e2 = nb.err;
            nb.freeAll();
            return cerr(e2, "push events");
        }
        std::vector<DevCell> keep(b->dcs);
        for (uint32_t c = 0; c < b->nCells; ++c) {
            b->dcs[c].evPtr = idx + b->synBase[c];
            b->dcs[c].evCur = idx + S + 1 + b->synBase[c];
            b->dcs[c].evTime = ev;
            b->dcs[c].evW = ev + m;
        }
        int rc = uploadDcs(b);
        if (rc != HS_OK) {
            b->dcs.swap(keep);
            nb.freeAll();
            return rc;
        }
        b->dEvOwnCur = idx + S + 1;
    } else {
        std::vector<uint32_t> curv(nptr.begin() + S + 1, nptr.end()), end(S), step(m);
        std::vector<float> act(m);
        for (uint32_t k = 0; k < S; ++k) end[k] = nptr[k + 1];
        for (size_t q = 0; q < m; ++q) {
            step[q] = deliveryStep(nt[q], b->clockDt);
            act[q] = (float)(nw[q] / b->clockDt);
        }
        uint32_t* dCur = nb.up(curv, b->st);
        const uint32_t* dEnd = nb.up(end, b->st);
        const uint32_t* dStep = nb.up(step, b->st);
        const float* dAct = nb.up(act, b->st);
        if (nb.err == cudaSuccess) nb.err = cudaStreamSynchronize(b->st);
        if (nb.err != cudaSuccess) {
            cudaError_t e2 = nb.err;
            nb.freeAll();
            return cerr(e2, "push events");
        }
        b->mb.evCur = dCur;
        b->dEvOwnCur = dCur;
        b->mb.evEnd = dEnd;
        b->mb.evStep = dStep;
        b->mb.evAct = dAct;
        if (b->gexec) {             // the graph holds the kernel's parameters
            cudaGraphExecDestroy(b->gexec);
            b->gexec = nullptr;
        }
    }
    b->evBuf.freeAll();
    b->evBuf = nb;
    nptr.resize((size_t)S + 1);
    b->evHostPtr.swap(nptr);
    b->evHostTime.swap(nt);
    b->evHostW.swap(nw);
    b->evOwned = true;
    b->pendSyn.clear();
    b->pendTime.clear();
    b->pendW.clear();
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
    if (e == cudaSuccess) {
        // keep freed pool memory for reuse instead of returning it at every
        // synchronisation (batches come and go in a serving loop)
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, b->device) == cudaSuccess) {
            uint64_t keep = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
        b->buf.st = b->packBuf.st = b->recBuf.st = b->injBuf.st = b->evBuf.st = b->st;
    }
    if (e != cudaSuccess) {
        delete b;
        return cerr(e, "batch stream");
    }
    if (precision == HS_PREC_MIXED) {
        b->threadsPerCta = 1024;
        b->ctasPerSm = 1;
    }
    if (tuning) {
        if (tuning->threads_per_cta) b->threadsPerCta = tuning->threads_per_cta;
        if (tuning->ctas_per_sm) b->ctasPerSm = tuning->ctas_per_sm;
        if (tuning->steps_per_launch) b->stepsPerLaunch = tuning->steps_per_launch;
        b->forestNodes = tuning->forest_nodes;
        b->maxCtas = tuning->max_ctas;
        if (tuning->elim_warps) b->elimWarps = tuning->elim_warps == 0xFFFFFFFFu ? 0 : tuning->elim_warps;
        if (tuning->wait_rounds) b->waitRounds = tuning->wait_rounds;
        if (tuning->cluster_ctas) b->clusterCtas = tuning->cluster_ctas;
        b->useGraph = tuning->use_graph != 0;
    }
    if (b->clusterCtas > 8 || (b->clusterCtas > 1 && precision != HS_PREC_MIXED)) {
        hs_batch_destroy(b);
        return berr(HS_EINVAL, "cluster_ctas: 1..8, mixed precision only");
    }
    const uint32_t maxTpc = precision == HS_PREC_FP64 ? 256 : 1024;
    if (b->threadsPerCta % 32 || b->threadsPerCta == 0 || b->threadsPerCta > maxTpc) {
        hs_batch_destroy(b);
        return berr(HS_EINVAL, "threads_per_cta must be a multiple of 32, at most 256 (FP64) or 1024 (mixed)");
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
    b->gatherBuf.freeAll();
    b->evBuf.freeAll();
    if (b->arena.base) cudaFreeAsync(b->arena.base, b->st);
    if (b->st) cudaStreamDestroy(b->st);
    delete b;
    return HS_OK;
}

int hs_batch_tune(HsBatch* b, const HsBatchTuning* t) {
    if (!b || !t) return berr(HS_EINVAL, "null argument");
    const uint32_t maxTpc = b->precision == HS_PREC_FP64 ? 256 : 1024;
    if (t->threads_per_cta) {
        if (t->threads_per_cta % 32 || t->threads_per_cta > maxTpc)
            return berr(HS_EINVAL, "threads_per_cta must be a multiple of 32, at most 256 (FP64) or 1024 (mixed)");
        b->threadsPerCta = t->threads_per_cta;
    }
    cudaError_t e = cudaStreamSynchronize(b->st);
    if (e != cudaSuccess) return cerr(e, "batch tune");
    const uint32_t cps = t->ctas_per_sm ? t->ctas_per_sm : b->ctasPerSm;
    const uint32_t ccl = t->cluster_ctas ? t->cluster_ctas : b->clusterCtas;
    if (ccl > 8 || (ccl > 1 && b->precision != HS_PREC_MIXED))
        return berr(HS_EINVAL, "cluster_ctas: 1..8, mixed precision only");
    const bool relayout = b->precision == HS_PREC_MIXED &&
                          (cps != b->ctasPerSm || t->forest_nodes != b->forestNodes || t->max_ctas != b->maxCtas ||
                           ccl != b->clusterCtas);
    b->clusterCtas = ccl;
    b->ctasPerSm = cps;
    b->forestNodes = t->forest_nodes;
    b->maxCtas = t->max_ctas;
    if (t->elim_warps) b->elimWarps = t->elim_warps == 0xFFFFFFFFu ? 0 : t->elim_warps;
    if (t->wait_rounds) b->waitRounds = t->wait_rounds;
    if (t->steps_per_launch) b->stepsPerLaunch = t->steps_per_launch;
    b->useGraph = t->use_graph != 0;
    if (relayout) {
        // a new forest packing renumbers every node: rebuild the layout; the
        // state, recording and inject targets start over
        if (b->gexec) {
            cudaGraphExecDestroy(b->gexec);
            b->gexec = nullptr;
        }
        dropRuntimeEvents(b);
        b->buf.freeAll();
        b->buf.err = cudaSuccess;
        b->recBuf.freeAll();
        b->recBuf.err = cudaSuccess;
        b->rec.clear();
        b->recBase = nullptr;
        b->injBuf.freeAll();
        b->injBuf.err = cudaSuccess;
        b->nInjTargets = 0;
        b->gatherBuf.freeAll();
        b->gatherBuf.err = cudaSuccess;
        b->dGatherVm = b->dGatherCa = nullptr;
        b->dGatherOut = nullptr;
        b->reinited = false;
        int rc = buildMixed(b);
        if (rc != HS_OK) return rc;
    }
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
    dropRuntimeEvents(b);
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
            evStep[e2] = deliveryStep(H.evTime[e2], clock_dt);
            evAct[e2] = (float)(H.evW[e2] / clock_dt);
        }
        if (!types.empty())
            e = cudaMemcpyAsync(b->dSynTypes, types.data(), types.size() * sizeof(SynType), cudaMemcpyHostToDevice,
                                b->st);
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
        // a timed-out wait invalidated the old state; the new one is valid
        if (e == cudaSuccess) e = cudaMemsetAsync(b->mb.err, 0, sizeof(uint32_t), b->st);
        if (e == cudaSuccess)
            e = launchBatchReinitMixed(b->mb, (uint32_t)H.nNodes, b->dMixInitVm, b->dMixC2dX0, b->dEvStart, b->st);
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
    if (int rc = flushRuntimeEvents(b)) return rc;
    const uint32_t K = b->stepsPerLaunch;
    if (b->evUsed >= 1024) {
        // fold the timings recorded so far, so that a long-running caller
        // that never asks for them keeps a bounded event list
        cudaError_t e0 = cudaStreamSynchronize(b->st);
        if (e0 != cudaSuccess) return cerr(e0, "batch process");
        for (size_t i = 0; i < b->evUsed; ++i) {
            float ms = 0;
            cudaEventElapsedTime(&ms, b->evs[i].first, b->evs[i].second);
            b->timedMs += ms;
            b->timedLaunches += 1;
        }
        b->evUsed = 0;
    }
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

int hs_batch_idle(HsBatch* b, int* idle) {
    if (!b || !idle) return berr(HS_EINVAL, "null argument");
    cudaError_t e = cudaStreamQuery(b->st);
    if (e == cudaSuccess) {
        *idle = 1;
        return HS_OK;
    }
    if (e == cudaErrorNotReady) {
        *idle = 0;
        return HS_OK;
    }
    return cerr(e, "batch query");
}

int hs_batch_sync(HsBatch* b) {
    if (!b) return berr(HS_EINVAL, "null batch");
    cudaError_t e = cudaStreamSynchronize(b->st);
    if (e != cudaSuccess) return cerr(e, "batch sync");
    if (b->precision == HS_PREC_MIXED && b->mb.err) {
        uint32_t flag = 0;
        e = cudaMemcpy(&flag, b->mb.err, 4, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cerr(e, "batch sync");
        if (flag)
            return berr(HS_ETIMEOUT, "a bounded wait of the split step gave up; results are invalid until reinit");
    }
    return HS_OK;
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
    if (n_ctas) *n_ctas = b->nCtas * (b->precision == HS_PREC_MIXED ? b->clusterCtas : 1);
    if (threads_per_cta) *threads_per_cta = b->threadsPerCta;
    if (steps_per_launch) *steps_per_launch = b->stepsPerLaunch;
    return HS_OK;
}

int hs_batch_forests(HsBatch* b, uint32_t* n_forests, uint32_t* n_shared) {
    if (!b) return berr(HS_EINVAL, "null batch");
    const bool mixed = b->precision == HS_PREC_MIXED;
    if (n_forests) *n_forests = mixed ? b->mh.nForests : 0;
    if (n_shared) *n_shared = mixed ? b->mh.nShared : 0;
    return HS_OK;
}

int hs_batch_set_stop_steps(HsBatch* b, const uint64_t* stop, uint32_t n) {
    if (!b || !stop) return berr(HS_EINVAL, "null argument");
    if (b->precision != HS_PREC_MIXED) return berr(HS_ENOTSUP, "stop steps are a mixed-batch feature");
    if (n != b->nCells) return berr(HS_EINVAL, "n must equal the number of cells");
    static_assert(sizeof(unsigned long long) == sizeof(uint64_t), "64-bit step counts");
    // per forest, the largest stop step of its cells: the kernel skips a
    // forest whose step count has reached it
    const size_t nF = b->forestCellPtr.empty() ? 0 : b->forestCellPtr.size() - 1;
    std::vector<unsigned long long> fstop(nF, 0);
    for (size_t f = 0; f < nF; ++f)
        for (uint32_t k = b->forestCellPtr[f]; k < b->forestCellPtr[f + 1]; ++k)
            fstop[f] = std::max<unsigned long long>(fstop[f], stop[b->forestCellIdx[k]]);
    cudaError_t e = cudaMemcpyAsync(b->dStopStep, stop, (size_t)n * 8, cudaMemcpyHostToDevice, b->st);
    if (e == cudaSuccess && nF)
        e = cudaMemcpyAsync(b->dForestStop, fstop.data(), nF * 8, cudaMemcpyHostToDevice, b->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
    if (e != cudaSuccess) return cerr(e, "stop steps");
    uint32_t any = 0;
    for (uint32_t c = 0; c < n; ++c) any |= stop[c] != UINT64_MAX;
    if (any != b->mb.anyStop) {
        // the flag is a kernel argument: a captured graph must be rebuilt
        b->mb.anyStop = any;
        if (b->gexec) {
            cudaGraphExecDestroy(b->gexec);
            b->gexec = nullptr;
        }
    }
    return HS_OK;
}

int hs_batch_read_steps(HsBatch* b, uint64_t* out, uint32_t n) {
    if (!b || !out) return berr(HS_EINVAL, "null argument");
    if (b->precision != HS_PREC_MIXED) return berr(HS_ENOTSUP, "per-cell step counts are a mixed-batch feature");
    if (n != b->nCells) return berr(HS_EINVAL, "n must equal the number of cells");
    cudaError_t e = cudaStreamSynchronize(b->st);
    if (e == cudaSuccess) e = cudaMemcpy(out, b->mb.stepCount, (size_t)n * 8, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? HS_OK : cerr(e, "read steps");
}

int hs_batch_read_spike_counts(HsBatch* b, uint32_t* out, uint32_t n) {
    if (!b || !out) return berr(HS_EINVAL, "null argument");
    if (b->precision != HS_PREC_MIXED) return berr(HS_ENOTSUP, "per-cell spike counts are a mixed-batch feature");
    if (n != b->nCells) return berr(HS_EINVAL, "n must equal the number of cells");
    cudaError_t e = cudaStreamSynchronize(b->st);
    if (e == cudaSuccess) e = cudaMemcpy(out, b->mb.spikeCount, (size_t)n * 4, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? HS_OK : cerr(e, "spike counts");
}

int hs_batch_poll(HsBatch* b, uint32_t first, uint32_t count, double* trace, uint64_t* steps,
                  uint32_t* spike_counts) {
    if (!b) return berr(HS_EINVAL, "null batch");
    if (b->precision != HS_PREC_MIXED) return berr(HS_ENOTSUP, "polling is a mixed-batch feature");
    cudaError_t e = cudaSuccess;
    if (count && trace) {
        if (b->rec.empty()) return berr(HS_ESTATE, "nothing is recorded");
        if ((uint64_t)first + count > b->recCap) return berr(HS_ECAPACITY, "window beyond the recording capacity");
        e = cudaMemcpyAsync(trace, b->recBase + (size_t)first * b->rec.size(), (size_t)count * b->rec.size() * 8,
                            cudaMemcpyDeviceToHost, b->st);
    }
    if (e == cudaSuccess && steps)
        e = cudaMemcpyAsync(steps, b->mb.stepCount, (size_t)b->nCells * 8, cudaMemcpyDeviceToHost, b->st);
    if (e == cudaSuccess && spike_counts)
        e = cudaMemcpyAsync(spike_counts, b->mb.spikeCount, (size_t)b->nCells * 4, cudaMemcpyDeviceToHost, b->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
    return e == cudaSuccess ? HS_OK : cerr(e, "batch poll");
}

int hs_batch_device_bytes(HsBatch* b, uint64_t* out) {
    if (!b || !out) return berr(HS_EINVAL, "null argument");
    *out = b->buf.bytes + b->packBuf.bytes + b->recBuf.bytes + b->injBuf.bytes + b->arena.size;
    return HS_OK;
}

int hs_batch_read_cell_spikes(HsBatch* b, uint32_t cell, uint32_t first, uint32_t* gen, double* time,
                              uint32_t capacity, uint32_t* n) {
    if (!b || !n) return berr(HS_EINVAL, "null argument");
    if (b->precision != HS_PREC_MIXED) return berr(HS_ENOTSUP, "per-cell spike reads are a mixed-batch feature");
    if (cell >= b->nCells) return berr(HS_EINVAL, "cell index out of range");
    cudaError_t e = cudaStreamSynchronize(b->st);
    uint32_t cnt = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&cnt, b->mb.spikeCount + cell, 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cerr(e, "cell spikes");
    *n = cnt;
    const uint32_t stored = std::min(cnt, b->spikeCap);
    const uint32_t k = first < stored ? std::min(stored - first, capacity) : 0;
    if (k && (gen || time)) {
        std::vector<uint32_t> g(k);
        std::vector<float> t(k);
        e = cudaMemcpy(g.data(), b->mb.spikeGen + (size_t)cell * b->spikeCap + first, k * 4, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess)
            e = cudaMemcpy(t.data(), b->mb.spikeTime + (size_t)cell * b->spikeCap + first, k * 4,
                           cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cerr(e, "cell spikes");
        for (uint32_t i = 0; i < k; ++i) {
            if (gen) gen[i] = g[i];
            if (time) time[i] = t[i];
        }
    }
    if (cnt > b->spikeCap) return berr(HS_ECAPACITY, "spike buffer overflow");
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
        // the cell's nodes lie inside one forest: copy their index range
        const std::vector<int64_t>& no = b->mh.nodeOf[cell];
        int64_t lo = INT64_MAX, hi = -1;
        for (int64_t g : no)
            if (g >= 0) {
                lo = std::min(lo, g);
                hi = std::max(hi, g);
            }
        std::vector<double> v(hi >= lo ? (size_t)(hi - lo + 1) : 0);
        if (e == cudaSuccess && !v.empty())
            e = cudaMemcpy(v.data(), b->mb.V + lo, v.size() * 8, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cerr(e, "batch read vm");
        for (uint32_t m = 0; m < n; ++m) out[m] = no[m] < 0 ? NAN : v[no[m] - lo];
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
        // the cell's pools are node-indexed inside one forest: one copy
        const std::vector<int64_t>& po = b->mh.poolOf[cell];
        int64_t lo = INT64_MAX, hi = -1;
        for (int64_t g : po)
            if (g >= 0) {
                lo = std::min(lo, g);
                hi = std::max(hi, g);
            }
        std::vector<float> v(hi >= lo ? (size_t)(hi - lo + 1) : 0);
        if (!v.empty()) e = cudaMemcpy(v.data(), b->mb.poolCa + lo, v.size() * 4, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cerr(e, "batch read ca");
        for (uint32_t m = 0; m < n; ++m) out[m] = po[m] < 0 ? NAN : (double)v[po[m] - lo];
    }
    return HS_OK;
}

int hs_batch_read_all(HsBatch* b, int field, double* out, uint64_t n) {
    if (!b || (!out && n)) return berr(HS_EINVAL, "null argument");
    if (field != HS_F_VM && field != HS_F_CA) return berr(HS_EINVAL, "field must be HS_F_VM or HS_F_CA");
    const bool vm = field == HS_F_VM;
    if (!b->nAllCompt && !b->nAllPool)
        for (const CellPlan& P : b->plans) {
            b->nAllCompt += P.hinesOf.size();
            b->nAllPool += P.poolSolverOf.size();
        }
    const uint64_t total = vm ? b->nAllCompt : b->nAllPool;
    if (n != total) return berr(HS_EINVAL, "n must equal the batch's total compartment (pool) count");
    if (!n) return HS_OK;
    const void**& list = vm ? b->dGatherVm : b->dGatherCa;
    b->gatherBuf.st = b->st;
    if (!list) {
        // device address of every value, cell after cell in model order
        std::vector<const void*> src;
        src.reserve(total);
        for (uint32_t c = 0; c < b->nCells; ++c) {
            const CellPlan& P = b->plans[c];
            if (vm) {
                for (size_t m = 0; m < P.hinesOf.size(); ++m) {
                    if (b->precision == HS_PREC_FP64)
                        src.push_back(P.hinesOf[m] < 0 ? nullptr : b->dcs[c].V + P.hinesOf[m]);
                    else
                        src.push_back(b->mh.nodeOf[c][m] < 0 ? nullptr : b->mb.V + b->mh.nodeOf[c][m]);
                }
            } else {
                for (size_t m = 0; m < P.poolSolverOf.size(); ++m) {
                    if (b->precision == HS_PREC_FP64)
                        src.push_back(P.poolSolverOf[m] < 0 ? nullptr : b->dcs[c].ca + P.poolSolverOf[m]);
                    else
                        src.push_back(b->mh.poolOf[c][m] < 0 ? nullptr : b->mb.poolCa + b->mh.poolOf[c][m]);
                }
            }
        }
        list = b->gatherBuf.up(src, b->st);
        if (!b->dGatherOut) b->dGatherOut = b->gatherBuf.alloc<double>(std::max(b->nAllCompt, b->nAllPool));
        if (b->gatherBuf.err != cudaSuccess) {
            cudaError_t e = b->gatherBuf.err;
            b->gatherBuf.freeAll();
            b->gatherBuf.err = cudaSuccess;
            b->dGatherVm = b->dGatherCa = nullptr;
            b->dGatherOut = nullptr;
            return cerr(e, "read all");
        }
    }
    const uint32_t f32 = (!vm && b->precision == HS_PREC_MIXED) ? 1u : 0u;
    cudaError_t e = launchGatherValues(list, f32, n, b->dGatherOut, b->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, b->dGatherOut, n * 8, cudaMemcpyDeviceToHost, b->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
    return e == cudaSuccess ? HS_OK : cerr(e, "read all");
}

int hs_batch_record(HsBatch* b, const uint32_t* cell, const uint32_t* compt, uint32_t n, uint32_t stride,
                    uint32_t capacity) {
    if (!b) return berr(HS_EINVAL, "null batch");
    if (n && (!cell || !compt || stride == 0 || capacity == 0)) return berr(HS_EINVAL, "bad recording request");
    // Every target is checked before the old recording is released, so a
    // rejected request leaves the previous recording in place.
    std::vector<std::vector<uint32_t>> per(b->nCells);
    for (uint32_t r = 0; r < n; ++r) {
        if (cell[r] >= b->nCells) return berr(HS_EINVAL, "recorded cell out of range");
        const CellPlan& P = b->plans[cell[r]];
        if (compt[r] >= P.hinesOf.size() || P.hinesOf[compt[r]] < 0)
            return berr(HS_EINVAL, "recorded compartment not in the cell");
        per[cell[r]].push_back(compt[r]);
    }
    cudaStreamSynchronize(b->st);
    if (b->gexec) {
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
    }
    b->recBuf.freeAll();
    b->recBuf.err = cudaSuccess;
    b->rec.clear();
    b->recBase = nullptr;
    // No recording until the new one is in place: the kernels never see the
    // freed buffers, even if an allocation below fails.
    for (DevCell& d : b->dcs) {
        d.nRec = 0;
        d.recCompt = nullptr;
        d.recBuf = nullptr;
    }
    for (MixCellRange& R : b->mh.cells) R.rec0 = R.nRec = 0;
    b->mb.recNode = nullptr;
    b->mb.recBuf = nullptr;
    b->mb.recLd = 0;
    auto cleared = [&](cudaError_t e0) -> int {
        cudaError_t e = cudaSuccess;
        if (b->precision == HS_PREC_FP64) {
            int rc = uploadDcs(b);
            if (rc) return rc;
        } else if (!b->mh.cells.empty()) {
            e = cudaMemcpyAsync((void*)b->mb.cells, b->mh.cells.data(),
                                b->mh.cells.size() * sizeof(MixCellRange), cudaMemcpyHostToDevice, b->st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
        }
        if (e0 != cudaSuccess) return cerr(e0, "batch record");
        return e == cudaSuccess ? HS_OK : cerr(e, "batch record");
    };
    if (!n) return cleared(cudaSuccess);
    b->recCap = capacity;
    b->recStride = stride;
    double* buf = b->recBuf.zeros<double>((size_t)n * capacity, b->st);
    if (b->recBuf.err != cudaSuccess) {
        cudaError_t e = b->recBuf.err;
        b->recBuf.freeAll();
        b->recBuf.err = cudaSuccess;
        return cleared(e);
    }
    uint32_t col = 0;
    if (b->precision == HS_PREC_FP64) {
        std::vector<uint32_t> hidx;
        std::vector<uint32_t> starts(b->nCells);
        std::vector<std::pair<uint32_t, uint32_t>> rec;
        for (uint32_t c = 0; c < b->nCells; ++c) {
            starts[c] = (uint32_t)hidx.size();
            for (uint32_t m : per[c]) {
                hidx.push_back((uint32_t)b->plans[c].hinesOf[m]);
                rec.push_back({c, m});
            }
        }
        uint32_t* didx = b->recBuf.up(hidx, b->st);
        if (b->recBuf.err != cudaSuccess) {
            cudaError_t e = b->recBuf.err;
            b->recBuf.freeAll();
            b->recBuf.err = cudaSuccess;
            return cleared(e);
        }
        for (uint32_t c = 0; c < b->nCells; ++c) {
            DevCell& d = b->dcs[c];
            d.nRec = (uint32_t)per[c].size();
            d.recStride = stride;
            d.recCap = capacity;
            d.recLd = n;
            d.recCompt = didx + starts[c];
            d.recBuf = buf + starts[c];
        }
        b->rec = std::move(rec);
        b->recBase = buf;
        return uploadDcs(b);
    }
    std::vector<uint32_t> nodes;
    std::vector<std::pair<uint32_t, uint32_t>> rec;
    for (uint32_t c = 0; c < b->nCells; ++c) {
        MixCellRange& R = b->mh.cells[c];
        R.rec0 = col;
        R.nRec = (uint32_t)per[c].size();
        for (uint32_t m : per[c]) {
            nodes.push_back((uint32_t)b->mh.nodeOf[c][m]);
            rec.push_back({c, m});
        }
        col += R.nRec;
    }
    uint32_t* dnodes = b->recBuf.up(nodes, b->st);
    if (b->recBuf.err != cudaSuccess) {
        cudaError_t e = b->recBuf.err;
        b->recBuf.freeAll();
        b->recBuf.err = cudaSuccess;
        for (MixCellRange& R : b->mh.cells) R.rec0 = R.nRec = 0;
        return cleared(e);
    }
    b->mb.recNode = dnodes;
    b->mb.recBuf = buf;
    b->mb.recLd = n;
    b->mb.recCap = capacity;
    b->mb.recStride = stride;
    b->rec = std::move(rec);
    b->recBase = buf;
    cudaError_t e = cudaMemcpyAsync((void*)b->mb.cells, b->mh.cells.data(), b->mh.cells.size() * sizeof(MixCellRange),
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

int hs_batch_set_inject_at(HsBatch* b, const uint32_t* cell, const uint32_t* compt, const double* values,
                           uint32_t n) {
    if (!b || (n && (!cell || !compt || !values))) return berr(HS_EINVAL, "null argument");
    if (n > kInjectWriteMax)
        return berr(HS_ECAPACITY, "hs_batch_set_inject_at takes at most 32768 writes per call");
    if (n == 0) return HS_OK;
    std::lock_guard<std::mutex> lock(injectStaticLock());
    InjectWrite* w = injectStaging();
    for (uint32_t k = 0; k < n; ++k) {
        if (cell[k] >= b->nCells) return berr(HS_EINVAL, "inject target cell out of range");
        const CellPlan& P = b->plans[cell[k]];
        if (compt[k] >= P.hinesOf.size() || P.hinesOf[compt[k]] < 0)
            return berr(HS_EINVAL, "inject target compartment not in the cell");
        if (b->precision == HS_PREC_FP64) {
            const uint32_t h = (uint32_t)P.hinesOf[compt[k]];
            w[k] = InjectWrite{b->dcs[cell[k]].injBasal + h, b->dcs[cell[k]].injPresent + h, values[k]};
        } else {
            const int32_t e = b->injEntryOf[cell[k]][compt[k]];
            if (e < 0) return berr(HS_ENOTSUP, "mixed batch: compartment had no inject or stimulus at setup");
            w[k] = InjectWrite{b->mb.injVal + e, nullptr, values[k]};
        }
    }
    int cur = -1;
    cudaError_t e = cudaGetDevice(&cur);
    if (e == cudaSuccess && cur != b->device) e = cudaSetDevice(b->device);
    if (e == cudaSuccess) e = scatterInjectStatic(b->device, n, b->st);
    if (cur >= 0 && cur != b->device) cudaSetDevice(cur);
    return e == cudaSuccess ? HS_OK : cerr(e, "set inject at");
}

int hs_batch_read_spikes(HsBatch* b, uint32_t* cell, uint32_t* gen, double* time, uint32_t capacity,
                         uint32_t* n) {
    if (!b || !n) return berr(HS_EINVAL, "null argument");
    cudaError_t e = cudaStreamSynchronize(b->st);
    if (e != cudaSuccess) return cerr(e, "batch spikes");
    // counts of every cell in one copy
    const uint32_t nC = b->nCells;
    DevBuf tmp;
    tmp.st = b->st;
    std::vector<uint32_t> cnt(nC);
    const uint32_t cap = b->spikeCap;
    if (b->precision == HS_PREC_FP64) {
        uint32_t* dcnt = tmp.alloc<uint32_t>(nC);
        e = tmp.err;
        if (e == cudaSuccess) e = launchSpikeCountsFp64(b->dDcs, nC, dcnt, b->st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(cnt.data(), dcnt, (size_t)nC * 4, cudaMemcpyDeviceToHost, b->st);
    } else {
        e = cudaMemcpyAsync(cnt.data(), b->mb.spikeCount, (size_t)nC * 4, cudaMemcpyDeviceToHost, b->st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
    if (e != cudaSuccess) {
        tmp.freeAll();
        return cerr(e, "batch spikes");
    }
    // the stored spikes of the cells that fit in `capacity`, gathered on the
    // device into one list and read with one copy per array
    std::vector<uint32_t> off(nC + 1, 0);
    uint64_t total = 0;
    bool overflow = false;
    for (uint32_t c = 0; c < nC; ++c) {
        const uint32_t m = std::min(cnt[c], cap);
        overflow |= cnt[c] > m;
        total += cnt[c];
        off[c + 1] = off[c] + m;
    }
    const uint32_t stored = off[nC];
    const uint32_t k = std::min(stored, capacity);
    if (k && (cell || gen || time)) {
        const uint32_t* doff = tmp.up(off, b->st);
        uint32_t* dgen = tmp.alloc<uint32_t>(stored);
        double* dtime = tmp.alloc<double>(stored);
        e = tmp.err;
        if (e == cudaSuccess)
            e = launchGatherSpikes(b->precision == HS_PREC_FP64 ? b->dDcs : nullptr, b->mb.spikeGen,
                                   b->mb.spikeTime, cap, nC, doff, dgen, dtime, b->st);
        if (e == cudaSuccess && gen) e = cudaMemcpyAsync(gen, dgen, (size_t)k * 4, cudaMemcpyDeviceToHost, b->st);
        if (e == cudaSuccess && time) e = cudaMemcpyAsync(time, dtime, (size_t)k * 8, cudaMemcpyDeviceToHost, b->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
        if (e == cudaSuccess && cell)
            for (uint32_t c = 0; c < nC && off[c] < k; ++c)
                for (uint32_t i = off[c]; i < off[c + 1] && i < k; ++i) cell[i] = c;
    }
    tmp.freeAll();
    if (e != cudaSuccess) return cerr(e, "batch spikes");
    *n = (uint32_t)std::min<uint64_t>(total, 0xFFFFFFFFu);
    if (overflow) return berr(HS_ECAPACITY, "a cell's spike buffer overflowed");
    return HS_OK;
}

}  // extern "C"

// The modulation field of HHChannels, HHChannel2Ds or SynChans of a batch,
// between process() calls: the zombie HHChannel's setModulation
// (HSolve::setHHmodulation, hsolve/HSolveInterface.cpp:445-451: values <= 0
// keep the old one) and the external channels' own field
// (ChanCommon::vSetModulation, biophysics/ChanCommon.cpp:46-49), as an
// Adaptor (signeur/Adaptor.cpp) writes it from a chemical model each step.
int hs_batch_push_events(HsBatch* b, const uint32_t* cell, const uint32_t* syn, const double* time,
                         const double* weight, uint32_t n) {
    if (!b) return berr(HS_EINVAL, "null batch");
    if (n == 0) return HS_OK;
    if (!cell || !syn || !time || !weight) return berr(HS_EINVAL, "null argument");
    for (uint32_t i = 0; i < n; ++i) {
        if (cell[i] >= b->nCells) return berr(HS_EINVAL, "event cell out of range");
        if (syn[i] >= b->plans[cell[i]].S) return berr(HS_EINVAL, "event SynChan index out of range");
        if (std::isnan(time[i])) return berr(HS_EINVAL, "event time is NaN");
    }
    const bool fp64 = b->precision == HS_PREC_FP64;
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t k = fp64 ? b->synBase[cell[i]] + syn[i] : (uint32_t)b->mh.synGlobal[cell[i]][syn[i]];
        b->pendSyn.push_back(k);
        b->pendTime.push_back(time[i]);
        b->pendW.push_back(weight[i]);
    }
    return HS_OK;
}

int hs_batch_set_modulation(HsBatch* b, int kind, const uint32_t* cell, const uint32_t* index, const double* value,
                            uint32_t n) {
    if (!b || (n && (!cell || !index || !value))) return berr(HS_EINVAL, "null argument");
    if (kind != HS_KIND_CHAN && kind != HS_KIND_CHAN2D && kind != HS_KIND_SYNCHAN)
        return berr(HS_EINVAL, "modulation: kind must be HS_KIND_CHAN, HS_KIND_CHAN2D or HS_KIND_SYNCHAN");
    const bool mixed = b->precision != HS_PREC_FP64;
    std::vector<ValueWrite> w;
    w.reserve(n);
    for (uint32_t k = 0; k < n; ++k) {
        if (cell[k] >= b->nCells) return berr(HS_EINVAL, "modulation: cell out of range");
        CellPlan& P = b->plans[cell[k]];
        const uint32_t c = cell[k], m = index[k];
        const double v = value[k];
        if (kind == HS_KIND_CHAN) {
            if (m >= P.chanSolverOf.size() || P.chanSolverOf[m] < 0)
                return berr(HS_EINVAL, "modulation: HHChannel not in the cell");
            if (!(v > 0.0)) continue;
            const uint32_t q = (uint32_t)P.chanSolverOf[m];
            P.modulation[q] = v;
            if (!mixed) {
                w.push_back({b->dcs[c].mod + q, v, 0, 0});
            } else {
                const int64_t sl = b->mh.chanSlot[c][m];
                if (sl < 0) return berr(HS_EINVAL, "modulation: HHChannel without a slot");
                float* gb = const_cast<float*>(b->mb.gbar) + (size_t)(sl % kMaxChan) * b->mb.ld + sl / kMaxChan;
                w.push_back({gb, P.Gbar[q] * v, 1, 0});
            }
        } else if (kind == HS_KIND_CHAN2D) {
            if (m >= P.K2) return berr(HS_EINVAL, "modulation: HHChannel2D not in the cell");
            P.c2dMod[m] = v;
            if (!mixed) {
                w.push_back({b->dcs[c].c2dMod + m, v, 0, 0});
            } else {
                const int64_t g = b->mh.c2dNode[c][m];
                if (g < 0) return berr(HS_EINVAL, "modulation: HHChannel2D without a node");
                w.push_back({const_cast<float*>(b->mb.k2gbar) + g, P.c2dGbar[m] * v, 1, 0});
            }
        } else {
            if (m >= P.S) return berr(HS_EINVAL, "modulation: SynChan not in the cell");
            P.synMod[m] = v;
            if (!mixed) {
                w.push_back({b->dcs[c].synMod + m, v, 0, 0});
            } else {
                const int64_t s = b->mh.synGlobal[c][m];
                if (s < 0) return berr(HS_EINVAL, "modulation: SynChan not in the layout");
                b->mh.synMod[s] = v;
                if (b->reinited) {          // norm (at the clock dt) x modulation, as reinit sets it
                    double xc1, xc2, yc1, yc2, nm;
                    synchanConstants(b->mh.synTau1[s], b->mh.synTau2[s], b->mh.synGbar[s], b->clockDt, &xc1,
                                     &xc2, &yc1, &yc2, &nm);
                    w.push_back({const_cast<float*>(b->mb.synNorm) + s, nm * v, 1, 0});
                }
            }
        }
    }
    if (w.empty()) return HS_OK;
    ValueWrite* d = nullptr;
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&d), w.size() * sizeof(ValueWrite), b->st);
    if (e != cudaSuccess) return cerr(e, "modulation");
    e = cudaMemcpyAsync(d, w.data(), w.size() * sizeof(ValueWrite), cudaMemcpyHostToDevice, b->st);
    if (e == cudaSuccess) e = launchScatterValues(d, (uint32_t)w.size(), b->st);
    cudaError_t f = cudaFreeAsync(d, b->st);
    if (e == cudaSuccess) e = f;
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);     // w is released on return
    return e == cudaSuccess ? HS_OK : cerr(e, "modulation");
}
