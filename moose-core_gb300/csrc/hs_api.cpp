// hs_api.cpp -- C ABI of the GB300 HSolve drop-in (include/moose_gb300.h).
//
// An HsSolver is one HSolve instance: its plan (host), one device arena with
// all per-cell arrays, and one CUDA stream.  Field access mirrors
// hsolve/HSolveInterface.cpp:66-533 including its quirks (setEm/setRm reset
// EmByRm to Em/Rm; setCm refreshes CmByDt with the current dt_; setRa only
// stores Ra; modulation ignores non-positive values).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <new>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/moose_gb300.h"
#include "hs_cell.h"
#include "hs_events.h"
#include "hs_plan.h"

using namespace hsg;

namespace {
thread_local std::string g_err;

int setErr(int code, const std::string& msg) {
    g_err = msg;
    return code;
}
int cudaErr(cudaError_t e, const char* where) {
    return setErr(HS_EDEVICE, std::string(where) + ": " + cudaGetErrorString(e));
}
}  // namespace

namespace hsg {
int setLastError(int code, const std::string& msg) { return setErr(code, msg); }
}  // namespace hsg

// The completion of one group launch (hs_process_group), shared by the
// solvers it stepped until each has ordered its own stream after it.
struct HsGroupDone {
    cudaEvent_t ev = nullptr;
    cudaStream_t st = nullptr;          // the stream the launch ran on
    ~HsGroupDone() {
        if (ev) cudaEventDestroy(ev);   // released once it has completed
    }
};

struct HsSolver {
    int device = 0;
    cudaStream_t st = nullptr;          // new work goes through stOf()
    // hs_process_group: the last group launch that stepped this solver on
    // another stream (work queued here next must wait for it); whether work
    // was queued on this stream since then (a group launch elsewhere must
    // wait for it, through evQueued)
    std::shared_ptr<HsGroupDone> group;
    bool queued = true;
    cudaEvent_t evQueued = nullptr;
    CellPlan P;
    Arena arena;
    DevCell dc;
    DevCell* dcDev = nullptr;    // device copy of dc (for the reinit kernel)
    double dt_ = 0;          // HSolve::dt_ (setup dt, clock dt after reinit)
    double clockDt = 0;
    bool reinited = false;
    int precision = HS_PREC_FP64;
    uint32_t clusterCtas = 0;    // CTAs stepping the cell (0: by its size)
    std::vector<double> initVm, injBasal;
    std::vector<uint8_t> injPresent;
    uint32_t* recCompt = nullptr;
    double* recBuf = nullptr;
    std::vector<uint32_t> recHost;
    // Runtime synaptic events (hs_push_events).  Until the first push the
    // kernel reads the description's events in the arena; after it, a
    // solver-owned copy holding the undelivered events of every SynChan,
    // merged in time order.  hostPtr/hostTime/hostW mirror that copy.
    std::vector<uint32_t> pendSyn;
    std::vector<double> pendTime, pendW;
    bool evOwned = false;
    std::vector<uint32_t> hostPtr;    // S+1 bounds, then S cursors (= the bounds)
    std::vector<double> hostTime, hostW;
    uint32_t* ownIdx = nullptr;       // device: evPtr (S+1), evCur (S)
    double* ownEv = nullptr;          // device: time (ownCap), weight (ownCap)
    size_t ownCap = 0;
    const uint32_t* descPtr = nullptr;
    uint32_t* descCur = nullptr;
    const double *descTime = nullptr, *descW = nullptr;
    // Field access mirror (see readDev/writeDev): host copies of arena
    // pages, valid while their epoch is the solver's; the epoch moves on
    // whenever device work may have changed the arena.  Writes wait in
    // `writes` (last one per address) until flushWrites scatters them.
    uint64_t epoch = 1;
    std::unordered_map<size_t, std::pair<uint64_t, std::vector<uint8_t>>> pages;
    std::map<uintptr_t, FieldWrite> writes;
    std::vector<FieldWrite> writeList;
    FieldWrite* dWrites = nullptr;
    size_t dWritesCap = 0;
};

namespace {

// The solver's stream for new work: it first waits for the group launch
// that last stepped the solver on another stream, and what it receives
// must come before the solver's next group launch.
cudaStream_t stOf(HsSolver* s) {
    if (s->group) {
        cudaStreamWaitEvent(s->st, s->group->ev, 0);
        s->group.reset();
    }
    s->queued = true;
    return s->st;
}

// ---- field access between process calls ------------------------------------
// The zombie get/set calls (hsolve/HSolveInterface.cpp) arrive one field at a
// time, typically many between two steps (a script reading every
// compartment's Vm, Tables polling, message destinations read-modify-writing
// their targets).  They are served from a host mirror of the solver's arena
// in pages of kPage bytes: a page is copied from the device on its first read
// after the device last ran; a write updates the mirror and is queued; the
// queue is applied by one scatter kernel before the next launch, before any
// page is copied again and before any direct device read.  So a burst of
// field reads costs one device round trip per page touched, and writes cost
// none until the next step.
constexpr size_t kPage = 64 * 1024;

// Applies the queued writes on the solver's stream (no wait: the launch or
// copy that needs them is queued behind the scatter).
int flushWrites(HsSolver* s) {
    if (s->writes.empty()) return HS_OK;
    s->writeList.clear();
    for (const auto& kv : s->writes) s->writeList.push_back(kv.second);
    const size_t n = s->writeList.size();
    if (n > s->dWritesCap) {
        // no scatter may still read the old list when it is freed
        if (s->dWrites) {
            cudaError_t e = cudaStreamSynchronize(stOf(s));
            if (e != cudaSuccess) return cudaErr(e, "field write");
            cudaFree(s->dWrites);
        }
        s->dWrites = nullptr;
        s->dWritesCap = 0;
        const size_t cap = std::max<size_t>(n, 256);
        cudaError_t e = cudaMalloc(&s->dWrites, cap * sizeof(FieldWrite));
        if (e != cudaSuccess) {
            s->dWrites = nullptr;
            return cudaErr(e, "field write");
        }
        s->dWritesCap = cap;
    }
    // the pageable source is staged by the copy call itself
    cudaError_t e = cudaMemcpyAsync(s->dWrites, s->writeList.data(), n * sizeof(FieldWrite),
                                    cudaMemcpyHostToDevice, stOf(s));
    if (e == cudaSuccess) e = launchScatterFields(s->dWrites, (uint32_t)n, stOf(s));
    if (e != cudaSuccess) return cudaErr(e, "field write");
    s->writes.clear();
    return HS_OK;
}

// Device work changed (or may have changed) the arena: every mirrored page
// is stale.
void arenaMoved(HsSolver* s) { ++s->epoch; }

// The arena page holding [a, a + n), or -1 when the range is not inside one
// page of the arena.
int64_t pageOf(const HsSolver* s, const void* p, size_t n) {
    const uintptr_t a = (uintptr_t)p, base = (uintptr_t)s->arena.base;
    if (!s->arena.base || a < base || a + n > base + s->arena.size) return -1;
    const size_t off = a - base;
    if (off / kPage != (off + n - 1) / kPage) return -1;
    return (int64_t)(off / kPage);
}

// The current host copy of arena page `idx`.
int mirrorPage(HsSolver* s, size_t idx, uint8_t** out) {
    auto& pg = s->pages[idx];
    if (pg.first != s->epoch) {
        int rc = flushWrites(s);
        if (rc) return rc;
        const size_t off = idx * kPage, n = std::min(kPage, s->arena.size - off);
        pg.second.resize(n);
        cudaError_t e = cudaMemcpyAsync(pg.second.data(), s->arena.base + off, n, cudaMemcpyDeviceToHost, stOf(s));
        if (e == cudaSuccess) e = cudaStreamSynchronize(stOf(s));
        if (e != cudaSuccess) {
            pg.first = 0;
            return cudaErr(e, "field read");
        }
        pg.first = s->epoch;
    }
    *out = pg.second.data();
    return HS_OK;
}

// Hands the pushed events to the device before a process call: the queue
// is rebuilt on the host (mergeEventQueue, hs_events.h) from the device
// cursors and uploaded to solver-owned arrays.  The step kernel is
// unchanged: it walks them exactly as it walks the description's events.
int flushEvents(HsSolver* s) {
    if (s->pendSyn.empty()) return HS_OK;
    const uint32_t S = s->P.S;
    std::vector<uint32_t> cur(S);
    cudaError_t e = cudaStreamSynchronize(stOf(s));
    if (e == cudaSuccess)
        e = cudaMemcpy(cur.data(), s->dc.evCur, S * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cudaErr(e, "push events");
    std::vector<uint32_t> nptr;
    std::vector<double> nt, nw;
    if (!mergeEventQueue(S, s->evOwned ? s->hostPtr : s->P.evPtr, s->evOwned ? s->hostTime : s->P.evTime,
                         s->evOwned ? s->hostW : s->P.evW, cur, s->pendSyn, s->pendTime, s->pendW, nptr, nt,
                         nw))
        return setErr(HS_ENOMEM, "too many queued synaptic events");
    const size_t m = nt.size();
    if (!s->ownIdx) {
        e = cudaMalloc(&s->ownIdx, nptr.size() * sizeof(uint32_t));
        if (e != cudaSuccess) {
            s->ownIdx = nullptr;
            return cudaErr(e, "push events");
        }
    }
    // a grown buffer replaces the old one only once it holds the new queue,
    // so that a failed allocation or copy leaves the solver's queue as it was
    double* ev = s->ownEv;
    size_t cap = s->ownCap;
    if (m > cap) {
        cap = std::max(m, 2 * cap);
        e = cudaMalloc(&ev, 2 * cap * sizeof(double));
        if (e != cudaSuccess) return cudaErr(e, "push events");
    }
    e = cudaMemcpyAsync(s->ownIdx, nptr.data(), nptr.size() * sizeof(uint32_t),
                        cudaMemcpyHostToDevice, stOf(s));
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ev, nt.data(), m * sizeof(double), cudaMemcpyHostToDevice, stOf(s));
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ev + cap, nw.data(), m * sizeof(double), cudaMemcpyHostToDevice, stOf(s));
    if (e == cudaSuccess) e = cudaStreamSynchronize(stOf(s));
    if (e != cudaSuccess) {
        if (ev != s->ownEv) cudaFree(ev);
        return cudaErr(e, "push events");
    }
    if (ev != s->ownEv && s->ownEv) cudaFree(s->ownEv);
    s->ownEv = ev;
    s->ownCap = cap;
    s->hostPtr.swap(nptr);
    s->hostTime.swap(nt);
    s->hostW.swap(nw);
    s->dc.evPtr = s->ownIdx;
    s->dc.evCur = s->ownIdx + S + 1;
    s->dc.evTime = s->ownEv;
    s->dc.evW = s->ownEv + s->ownCap;
    s->evOwned = true;
    s->pendSyn.clear();
    s->pendTime.clear();
    s->pendW.clear();
    return HS_OK;
}

}  // namespace

extern "C" {

const char* hs_last_error(void) { return g_err.c_str(); }

int hs_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

const char* hs_build_info(void) {
    return "moose_gb300 HSolve: sm_103a; FP64 kernels built with --fmad=false";
}

int hs_create(const HsCellDesc* cell, uint32_t seed, double dt, int precision, HsSolver** out) {
    if (!cell || !out) return setErr(HS_EINVAL, "null argument");
    *out = nullptr;
    if (precision != HS_PREC_FP64)
        return setErr(HS_ENOTSUP, "the drop-in solver runs FP64; mixed precision is a batch option");
    HsSolver* s = new (std::nothrow) HsSolver();
    if (!s) return setErr(HS_ENOMEM, "host allocation failed");
    std::string err;
    try {
        if (!buildPlan(*cell, seed, dt, s->P, err)) {
            delete s;
            return setErr(HS_EINVAL, err);
        }
    } catch (const std::bad_alloc&) {
        delete s;
        return setErr(HS_ENOMEM, "host allocation failed during setup");
    } catch (...) {
        delete s;
        return setErr(HS_EINVAL, "setup failed");
    }
    if (hs_device_count() == 0) {
        delete s;
        return setErr(HS_EDEVICE, "no CUDA device");
    }
    cudaError_t e = cudaGetDevice(&s->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete s;
        return cudaErr(e, "stream");
    }
    const uint32_t spikeCap = 1u << 16;
    Arena dry;
    layoutCell(s->P, dry, s->dc, spikeCap, stOf(s));
    dry.take<DevCell>(1);
    s->arena.size = dry.used + 256;
    e = cudaMalloc(&s->arena.base, s->arena.size);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->arena.base, 0, s->arena.size, stOf(s));
    if (e == cudaSuccess) e = layoutCell(s->P, s->arena, s->dc, spikeCap, stOf(s));
    s->dcDev = s->arena.take<DevCell>(1);
    s->descPtr = s->dc.evPtr;
    s->descCur = s->dc.evCur;
    s->descTime = s->dc.evTime;
    s->descW = s->dc.evW;
    if (e == cudaSuccess) e = cudaStreamSynchronize(stOf(s));
    if (e != cudaSuccess) {
        int rc = cudaErr(e, "device setup");
        hs_destroy(s);
        return rc;
    }
    s->dt_ = dt;
    s->dc.dt = dt;
    s->precision = precision;
    s->initVm = s->P.initVm;
    s->injBasal = s->P.injBasal;
    s->injPresent = s->P.injPresent;
    *out = s;
    return HS_OK;
}

int hs_destroy(HsSolver* s) {
    if (!s) return HS_OK;
    if (s->st) cudaStreamSynchronize(stOf(s));
    if (s->arena.base) cudaFree(s->arena.base);
    if (s->recCompt) cudaFree(s->recCompt);
    if (s->recBuf) cudaFree(s->recBuf);
    if (s->ownIdx) cudaFree(s->ownIdx);
    if (s->ownEv) cudaFree(s->ownEv);
    if (s->dWrites) cudaFree(s->dWrites);
    if (s->evQueued) cudaEventDestroy(s->evQueued);
    if (s->st) cudaStreamDestroy(s->st);
    delete s;
    return HS_OK;
}

int hs_reinit(HsSolver* s, double clock_dt) {
    if (!s) return setErr(HS_EINVAL, "null solver");
    if (!(clock_dt > 0)) return setErr(HS_EINVAL, "clock dt must be positive");
    s->dt_ = clock_dt;            // HSolve::reinit: dt_ = p->dt
    s->clockDt = clock_dt;
    s->dc.dt = clock_dt;
    // SimpleSynHandler::vReinit empties the queue; the description's events
    // are queued again (the reinit kernel rewinds their cursors).
    s->pendSyn.clear();
    s->pendTime.clear();
    s->pendW.clear();
    if (s->evOwned) {
        s->dc.evPtr = s->descPtr;
        s->dc.evCur = s->descCur;
        s->dc.evTime = s->descTime;
        s->dc.evW = s->descW;
        s->evOwned = false;
    }
    std::vector<double> sc(5 * (size_t)s->P.S + 1);
    synConsts(s->P, clock_dt, sc.data());
    int rc = flushWrites(s);
    if (rc) return rc;
    arenaMoved(s);
    cudaError_t e = cudaMemcpyAsync((void*)s->dc.synConst, sc.data(), 5 * (size_t)s->P.S * 8,
                                    cudaMemcpyHostToDevice, stOf(s));
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->dc.initVm, s->initVm.data(), s->P.N * 8, cudaMemcpyHostToDevice, stOf(s));
    if (e == cudaSuccess) e = cudaMemcpyAsync(s->dcDev, &s->dc, sizeof(DevCell), cudaMemcpyHostToDevice, stOf(s));
    if (e == cudaSuccess) e = launchReinitFp64(s->dcDev, 1, stOf(s));
    if (e == cudaSuccess) e = cudaStreamSynchronize(stOf(s));
    if (e != cudaSuccess) return cudaErr(e, "reinit");
    s->reinited = true;
    return HS_OK;
}

// CTAs that step a solver's cell: the size rule unless set.  A cell's step
// on one CTA is bound by one SM's FP64 issue of its channel and matrix-row
// work (~1 us per step per 2 compartments on GB300); from kClusterRows
// compartments on, a cluster of up to 8 CTAs shares that work (the
// elimination, a few dozen levels, stays on one CTA).
constexpr uint32_t kClusterRows = 1024;

uint32_t stepCtas(const HsSolver* s) {
    if (s->clusterCtas) return s->clusterCtas;
    const uint32_t n = s->P.N;
    if (n < kClusterRows) return 1;
    return std::min<uint32_t>(8, n / (kClusterRows / 2));
}

int hs_set_cluster_ctas(HsSolver* s, uint32_t ctas) {
    if (!s) return setErr(HS_EINVAL, "null solver");
    if (ctas > 8) return setErr(HS_EINVAL, "cluster_ctas: 0 (by cell size) or 1..8");
    s->clusterCtas = ctas;
    return HS_OK;
}

int hs_get_cluster_ctas(HsSolver* s, uint32_t* out) {
    if (!s || !out) return setErr(HS_EINVAL, "null argument");
    *out = stepCtas(s);
    return HS_OK;
}

int hs_process(HsSolver* s, uint32_t nsteps) {
    if (!s) return setErr(HS_EINVAL, "null solver");
    if (!s->reinited) return setErr(HS_ESTATE, "reinit before process");
    if (nsteps == 0) return HS_OK;
    int rc = flushEvents(s);
    if (!rc) rc = flushWrites(s);
    if (rc) return rc;
    arenaMoved(s);
    const uint32_t ctas = stepCtas(s);
    cudaError_t e = ctas > 1 ? launchStepFp64Cluster(s->dc, ctas, nsteps, stOf(s))
                             : launchStepFp64(s->dc, nsteps, stOf(s));
    if (e != cudaSuccess) return cudaErr(e, "process");
    return HS_OK;
}

int hs_process_group(HsSolver* const* solvers, uint32_t n, uint32_t nsteps) {
    if (n == 0) return HS_OK;
    if (!solvers) return setErr(HS_EINVAL, "null argument");
    for (uint32_t k = 0; k < n; ++k) {
        if (!solvers[k]) return setErr(HS_EINVAL, "null solver");
        if (!solvers[k]->reinited) return setErr(HS_ESTATE, "reinit before process");
        if (solvers[k]->device != solvers[0]->device)
            return setErr(HS_EINVAL, "the solvers of a group must be on one device");
        for (uint32_t j = 0; j < k; ++j)
            if (solvers[j] == solvers[k]) return setErr(HS_EINVAL, "a solver appears twice in the group");
    }
    if (nsteps == 0) return HS_OK;
    // members by the CTAs that step them: one launch per class, on the
    // stream of the class's first member (the clusters first: they need
    // whole free SM groups)
    std::vector<std::vector<uint32_t>> cls(9);
    for (uint32_t k = 0; k < n; ++k) {
        HsSolver* s = solvers[k];
        int rc = flushEvents(s);
        if (!rc) rc = flushWrites(s);
        if (rc) return rc;
        arenaMoved(s);
        cls[stepCtas(s)].push_back(k);
    }
    cudaError_t e = cudaSuccess;
    for (uint32_t ctas = 8; ctas >= 1 && e == cudaSuccess; --ctas) {
        const std::vector<uint32_t>& m = cls[ctas];
        if (m.empty()) continue;
        cudaStream_t gst = solvers[m[0]]->st;
        // The launch follows each member's work: what was queued on its own
        // stream since its last group launch (an event there) and the
        // group launch that last stepped it on another stream.  A group
        // that repeats on the same streams, with nothing queued between
        // its calls, needs neither: stream order covers it.
        std::vector<DevCell> cells(m.size());
        for (size_t k = 0; k < m.size() && e == cudaSuccess; ++k) {
            HsSolver* s = solvers[m[k]];
            cells[k] = s->dc;
            if (s->st != gst && s->queued) {
                if (!s->evQueued) e = cudaEventCreateWithFlags(&s->evQueued, cudaEventDisableTiming);
                if (e == cudaSuccess) e = cudaEventRecord(s->evQueued, s->st);
                if (e == cudaSuccess) e = cudaStreamWaitEvent(gst, s->evQueued, 0);
            }
            if (e == cudaSuccess && s->group && s->group->st != gst) e = cudaStreamWaitEvent(gst, s->group->ev, 0);
        }
        DevCell* dCells = nullptr;
        if (e == cudaSuccess) e = cudaMallocAsync(&dCells, m.size() * sizeof(DevCell), gst);
        // (a copy from pageable memory has read `cells` when it returns)
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(dCells, cells.data(), m.size() * sizeof(DevCell), cudaMemcpyHostToDevice, gst);
        if (e == cudaSuccess) e = launchGroupStepFp64(dCells, (uint32_t)m.size(), ctas, nsteps, gst);
        if (dCells) cudaFreeAsync(dCells, gst);
        auto done = std::make_shared<HsGroupDone>();
        done->st = gst;
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&done->ev, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(done->ev, gst);
        if (e != cudaSuccess) break;
        // the members' next work waits for the launch (stOf); the first
        // member's stream holds it already
        for (size_t k = 0; k < m.size(); ++k) {
            HsSolver* s = solvers[m[k]];
            if (s->st == gst) {
                s->group.reset();
                s->queued = true;
            } else {
                s->group = done;
                s->queued = false;
            }
        }
    }
    if (e != cudaSuccess) return cudaErr(e, "process group");
    return HS_OK;
}

int hs_sync(HsSolver* s) {
    if (!s) return setErr(HS_EINVAL, "null solver");
    if (int rc = flushWrites(s)) return rc;
    cudaError_t e = cudaStreamSynchronize(stOf(s));
    if (e != cudaSuccess) return cudaErr(e, "sync");
    return HS_OK;
}

int hs_set_ca_advance(HsSolver* s, int v) {
    if (!s) return setErr(HS_EINVAL, "null solver");
    if (v != 0 && v != 1) return setErr(HS_EINVAL, "HSolve: caAdvance should be either 0 or 1");
    s->dc.caAdvance = v;
    return HS_OK;
}

int hs_get_ca_advance(HsSolver* s, int* out) {
    if (!s || !out) return setErr(HS_EINVAL, "null argument");
    *out = s->dc.caAdvance;
    return HS_OK;
}

int hs_get_table_grid(HsSolver* s, double* vmin, double* vmax, int* vdiv, double* camin,
                      double* camax, int* cadiv) {
    if (!s) return setErr(HS_EINVAL, "null solver");
    if (vmin) *vmin = s->P.vMin;
    if (vmax) *vmax = s->P.vMax;
    if (vdiv) *vdiv = s->P.vDiv;
    if (camin) *camin = s->P.caMin;
    if (camax) *camax = s->P.caMax;
    if (cadiv) *cadiv = s->P.caDiv;
    return HS_OK;
}

int hs_get_nsteps(HsSolver* s, uint64_t* out) {
    if (!s || !out) return setErr(HS_EINVAL, "null argument");
    if (int rc = flushWrites(s)) return rc;
    DevCtl ctl;
    cudaError_t e = cudaMemcpyAsync(&ctl, s->dc.ctl, sizeof(ctl), cudaMemcpyDeviceToHost, stOf(s));
    if (e == cudaSuccess) e = cudaStreamSynchronize(stOf(s));
    if (e != cudaSuccess) return cudaErr(e, "get nsteps");
    *out = ctl.nSteps;
    return HS_OK;
}

}  // extern "C"

namespace {

// One field value through the mirror (every field lives in the arena).
template <class T>
int readDev(HsSolver* s, const T* p, T* out) {
    const int64_t idx = pageOf(s, p, sizeof(T));
    if (idx < 0) {
        int rc = flushWrites(s);
        if (rc) return rc;
        cudaError_t e = cudaMemcpyAsync(out, p, sizeof(T), cudaMemcpyDeviceToHost, stOf(s));
        if (e == cudaSuccess) e = cudaStreamSynchronize(stOf(s));
        return e == cudaSuccess ? HS_OK : cudaErr(e, "field read");
    }
    uint8_t* pg;
    int rc = mirrorPage(s, (size_t)idx, &pg);
    if (rc) return rc;
    std::memcpy(out, pg + ((const uint8_t*)p - (const uint8_t*)s->arena.base - (size_t)idx * kPage), sizeof(T));
    return HS_OK;
}
template <class T>
int writeDev(HsSolver* s, T* p, T v) {
    static_assert(sizeof(T) == 1 || sizeof(T) == 4 || sizeof(T) == 8, "field write size");
    const int64_t idx = pageOf(s, p, sizeof(T));
    if (idx < 0 || ((uintptr_t)p % sizeof(T)) != 0) {
        int rc = flushWrites(s);
        if (rc) return rc;
        cudaError_t e = cudaMemcpyAsync(p, &v, sizeof(T), cudaMemcpyHostToDevice, stOf(s));
        if (e == cudaSuccess) e = cudaStreamSynchronize(stOf(s));
        arenaMoved(s);
        return e == cudaSuccess ? HS_OK : cudaErr(e, "field write");
    }
    FieldWrite w{p, 0ull, (uint32_t)sizeof(T), 0u};
    std::memcpy(&w.bits, &v, sizeof(T));
    s->writes[(uintptr_t)p] = w;
    auto it = s->pages.find((size_t)idx);
    if (it != s->pages.end() && it->second.first == s->epoch)
        std::memcpy(it->second.second.data() + ((uint8_t*)p - (uint8_t*)s->arena.base - (size_t)idx * kPage), &v,
                    sizeof(T));
    return HS_OK;
}

int comptIndex(HsSolver* s, uint32_t m, uint32_t* h) {
    if (m >= s->P.hinesOf.size() || s->P.hinesOf[m] < 0)
        return setErr(HS_EINVAL, "compartment is not handled by this solver");
    *h = (uint32_t)s->P.hinesOf[m];
    return HS_OK;
}
int chanIndex(HsSolver* s, uint32_t m, uint32_t* q) {
    if (m >= s->P.chanSolverOf.size() || s->P.chanSolverOf[m] < 0)
        return setErr(HS_EINVAL, "channel is not handled by this solver");
    *q = (uint32_t)s->P.chanSolverOf[m];
    return HS_OK;
}
int poolIndex(HsSolver* s, uint32_t m, uint32_t* p) {
    if (m >= s->P.poolSolverOf.size() || s->P.poolSolverOf[m] < 0)
        return setErr(HS_EINVAL, "pool is not handled by this solver");
    *p = (uint32_t)s->P.poolSolverOf[m];
    return HS_OK;
}
// state index of gate w (0 X, 1 Y, 2 Z) of solver channel q, or -1
int64_t gateState(HsSolver* s, uint32_t q, int w) {
    double pw[3] = {s->P.Xpow[q], s->P.Ypow[q], s->P.Zpow[q]};
    if (pw[w] == 0.0) return -1;
    int64_t k = s->P.stateOff[q];
    for (int i = 0; i < w; ++i) if (pw[i] > 0.0) ++k;
    return k;
}

}  // namespace

extern "C" {

int hs_get_field(HsSolver* s, int kind, int field, uint32_t index, double* out) {
    if (!s || !out) return setErr(HS_EINVAL, "null argument");
    uint32_t i;
    int rc;
    const CellPlan& P = s->P;
    switch (kind) {
    case HS_KIND_COMPT:
        if ((rc = comptIndex(s, index, &i))) return rc;
        switch (field) {
        case HS_F_VM: return readDev(s, s->dc.V + i, out);
        case HS_F_CM: *out = P.Cm[i]; return HS_OK;
        case HS_F_EM: *out = P.Em[i]; return HS_OK;
        case HS_F_RM: *out = P.Rm[i]; return HS_OK;
        case HS_F_RA: *out = P.Ra[i]; return HS_OK;
        case HS_F_INITVM: *out = s->initVm[i]; return HS_OK;
        case HS_F_INJECT: {
            uint8_t present;
            if ((rc = readDev(s, s->dc.injPresent + i, &present))) return rc;
            if (!present) { *out = 0.0; return HS_OK; }
            return readDev(s, s->dc.injBasal + i, out);
        }
        case HS_F_IM: {   // HSolve::getIm (hsolve/HSolveInterface.cpp:161-182)
            double V, EmByRm, pg, pge;
            if ((rc = readDev(s, s->dc.V + i, &V)) || (rc = readDev(s, s->dc.EmByRm + i, &EmByRm)) ||
                (rc = readDev(s, s->dc.prevExt + 2 * i, &pg)) || (rc = readDev(s, s->dc.prevExt + 2 * i + 1, &pge)))
                return rc;
            double Im = EmByRm - V / P.Rm[i];
            for (uint32_t q = P.chanPtr[i]; q < P.chanPtr[i + 1]; ++q) {
                double gk, ek;
                if ((rc = readDev(s, s->dc.Gk + q, &gk)) || (rc = readDev(s, s->dc.Ek + q, &ek))) return rc;
                Im += (ek - V) * gk;
            }
            Im += pge - pg * V;
            *out = Im;
            return HS_OK;
        }
        }
        return setErr(HS_EINVAL, "unknown compartment field");
    case HS_KIND_CHAN: {
        if ((rc = chanIndex(s, index, &i))) return rc;
        int64_t k;
        switch (field) {
        case HS_F_GBAR: return readDev(s, s->dc.Gbar + i, out);
        case HS_F_EK: return readDev(s, s->dc.Ek + i, out);
        case HS_F_GK: return readDev(s, s->dc.Gk + i, out);
        case HS_F_IK: {
            double gk, ek, V;
            if ((rc = readDev(s, s->dc.Gk + i, &gk)) || (rc = readDev(s, s->dc.Ek + i, &ek))) return rc;
            uint32_t ic = 0;
            while (P.chanPtr[ic + 1] <= i) ++ic;
            if ((rc = readDev(s, s->dc.V + ic, &V))) return rc;
            *out = (ek - V) * gk;
            return HS_OK;
        }
        case HS_F_X: case HS_F_Y: case HS_F_Z:
            k = gateState(s, i, field - HS_F_X);
            if (k < 0) { *out = 0.0; return HS_OK; }
            return readDev(s, s->dc.state + k, out);
        case HS_F_INSTANT: {
            int32_t v;
            if ((rc = readDev(s, s->dc.instant + i, &v))) return rc;
            *out = v;
            return HS_OK;
        }
        case HS_F_MODULATION: return readDev(s, s->dc.mod + i, out);
        case HS_F_XPOWER: return readDev(s, s->dc.Xpow + i, out);
        case HS_F_YPOWER: return readDev(s, s->dc.Ypow + i, out);
        case HS_F_ZPOWER: return readDev(s, s->dc.Zpow + i, out);
        }
        return setErr(HS_EINVAL, "unknown channel field");
    }
    case HS_KIND_POOL:
        if ((rc = poolIndex(s, index, &i))) return rc;
        switch (field) {
        case HS_F_CA: return readDev(s, s->dc.ca + i, out);
        case HS_F_CABASAL: return readDev(s, s->dc.CaBasal + i, out);
        case HS_F_CEILING: return readDev(s, s->dc.ceil + i, out);
        case HS_F_FLOOR: return readDev(s, s->dc.floor_ + i, out);
        }
        return setErr(HS_EINVAL, "unknown pool field");
    case HS_KIND_CHAN2D:
        if (index >= P.K2) return setErr(HS_EINVAL, "HHChannel2D index out of range");
        if (field == HS_F_X) return readDev(s, s->dc.c2dX + index, out);
        if (field == HS_F_GK) return readDev(s, s->dc.c2dGk + index, out);
        if (field == HS_F_GBAR) return readDev(s, s->dc.c2dGbar + index, out);
        if (field == HS_F_EK) return readDev(s, s->dc.c2dEk + index, out);
        return setErr(HS_EINVAL, "unknown HHChannel2D field");
    case HS_KIND_SYNCHAN:
        if (index >= P.S) return setErr(HS_EINVAL, "SynChan index out of range");
        if (field == HS_F_GK) return readDev(s, s->dc.synGk + index, out);
        if (field == HS_F_X) return readDev(s, s->dc.synX + index, out);
        if (field == HS_F_Y) return readDev(s, s->dc.synY + index, out);
        if (field == HS_F_EK) return readDev(s, s->dc.synEk + index, out);
        return setErr(HS_EINVAL, "unknown SynChan field");
    }
    return setErr(HS_EINVAL, "unknown object kind");
}

int hs_set_field(HsSolver* s, int kind, int field, uint32_t index, double value) {
    if (!s) return setErr(HS_EINVAL, "null solver");
    uint32_t i;
    int rc;
    CellPlan& P = s->P;
    switch (kind) {
    case HS_KIND_COMPT:
        if ((rc = comptIndex(s, index, &i))) return rc;
        switch (field) {
        case HS_F_VM: return writeDev(s, s->dc.V + i, value);
        case HS_F_CM:
            P.Cm[i] = value;
            return writeDev(s, s->dc.CmByDt + i, 2.0 * value / s->dt_);
        case HS_F_EM:
            P.Em[i] = value;
            return writeDev(s, s->dc.EmByRm + i, value / P.Rm[i]);
        case HS_F_RM:
            P.Rm[i] = value;
            return writeDev(s, s->dc.EmByRm + i, P.Em[i] / value);
        case HS_F_RA: P.Ra[i] = value; return HS_OK;
        case HS_F_INITVM: s->initVm[i] = value; return HS_OK;   // used at the next reinit
        case HS_F_INJECT:
            s->injBasal[i] = value;
            s->injPresent[i] = 1;
            if ((rc = writeDev<uint8_t>(s, s->dc.injPresent + i, 1))) return rc;
            return writeDev(s, s->dc.injBasal + i, value);
        }
        return setErr(HS_EINVAL, "compartment field not writable");
    case HS_KIND_CHAN: {
        if ((rc = chanIndex(s, index, &i))) return rc;
        int64_t k;
        switch (field) {
        case HS_F_GBAR: return writeDev(s, s->dc.Gbar + i, value);
        case HS_F_EK: return writeDev(s, s->dc.Ek + i, value);
        case HS_F_GK: return writeDev(s, s->dc.Gk + i, value);
        case HS_F_X: case HS_F_Y: case HS_F_Z:
            k = gateState(s, i, field - HS_F_X);
            if (k < 0) return HS_OK;
            return writeDev(s, s->dc.state + k, value);
        case HS_F_INSTANT: return writeDev<int32_t>(s, s->dc.instant + i, (int32_t)value);
        case HS_F_MODULATION:
            if (value > 0.0) return writeDev(s, s->dc.mod + i, value);
            return HS_OK;
        }
        return setErr(HS_EINVAL, "channel field not writable");
    }
    case HS_KIND_POOL: {
        if ((rc = poolIndex(s, index, &i))) return rc;
        double basal, cc;
        switch (field) {
        case HS_F_CA:   // HSolve::setCa: ca_ = Ca, c_ = Ca - CaBasal_
            if ((rc = readDev(s, s->dc.CaBasal + i, &basal))) return rc;
            if ((rc = writeDev(s, s->dc.ca + i, value))) return rc;
            return writeDev(s, s->dc.c + i, value - basal);
        case HS_F_CABASAL:   // CaConcStruct::setCaBasal keeps Ca
            if ((rc = readDev(s, s->dc.CaBasal + i, &basal)) || (rc = readDev(s, s->dc.c + i, &cc))) return rc;
            if ((rc = writeDev(s, s->dc.c + i, cc + (basal - value)))) return rc;
            return writeDev(s, s->dc.CaBasal + i, value);
        case HS_F_CEILING: return writeDev(s, s->dc.ceil + i, value);
        case HS_F_FLOOR: return writeDev(s, s->dc.floor_ + i, value);
        }
        return setErr(HS_EINVAL, "pool field not writable");
    }
    case HS_KIND_CHAN2D:
        if (index >= P.K2) return setErr(HS_EINVAL, "HHChannel2D index out of range");
        if (field == HS_F_GBAR) return writeDev(s, s->dc.c2dGbar + index, value);
        if (field == HS_F_EK) return writeDev(s, s->dc.c2dEk + index, value);
        if (field == HS_F_MODULATION) return writeDev(s, s->dc.c2dMod + index, value);
        return setErr(HS_EINVAL, "HHChannel2D field not writable");
    case HS_KIND_SYNCHAN:
        if (index >= P.S) return setErr(HS_EINVAL, "SynChan index out of range");
        if (field == HS_F_EK) return writeDev(s, s->dc.synEk + index, value);
        if (field == HS_F_MODULATION) return writeDev(s, s->dc.synMod + index, value);
        return setErr(HS_EINVAL, "SynChan field not writable");
    }
    return setErr(HS_EINVAL, "unknown object kind");
}

int hs_set_tau_b(HsSolver* s, uint32_t pool, double tau, double B) {
    if (!s) return setErr(HS_EINVAL, "null solver");
    uint32_t i;
    int rc;
    if ((rc = poolIndex(s, pool, &i))) return rc;
    if (!(tau != 0.0)) return setErr(HS_EINVAL, "tau must be non-zero");
    double dt = s->dt_;   // CaConcStruct::setTauB with HSolve::dt_
    if ((rc = writeDev(s, s->dc.f1 + i, 4.0 / (2.0 + dt / tau) - 1.0))) return rc;
    return writeDev(s, s->dc.f2 + i, 2.0 * B * dt / (2.0 + dt / tau));
}

int hs_add_inject(HsSolver* s, uint32_t compt, double value) {
    if (!s) return setErr(HS_EINVAL, "null solver");
    uint32_t i;
    int rc;
    if ((rc = comptIndex(s, compt, &i))) return rc;
    double cur;
    if ((rc = readDev(s, s->dc.injVarying + i, &cur))) return rc;
    s->injPresent[i] = 1;
    if ((rc = writeDev<uint8_t>(s, s->dc.injPresent + i, 1))) return rc;
    return writeDev(s, s->dc.injVarying + i, cur + value);
}

int hs_add_gkek(HsSolver* s, uint32_t compt, double Gk, double Ek) {
    if (!s) return setErr(HS_EINVAL, "null solver");
    uint32_t i;
    int rc;
    if ((rc = comptIndex(s, compt, &i))) return rc;
    double g, ge;
    if ((rc = readDev(s, s->dc.ext + 2 * i, &g)) || (rc = readDev(s, s->dc.ext + 2 * i + 1, &ge))) return rc;
    if ((rc = writeDev(s, s->dc.ext + 2 * i, g + Gk))) return rc;
    return writeDev(s, s->dc.ext + 2 * i + 1, ge + Gk * Ek);
}

int hs_add_conc(HsSolver* s, uint32_t chan, double conc) {
    if (!s) return setErr(HS_EINVAL, "null solver");
    uint32_t q;
    int rc;
    if ((rc = chanIndex(s, chan, &q))) return rc;
    return writeDev(s, s->dc.extCa + q, conc);
}

int hs_add_ica(HsSolver* s, uint32_t pool, double ica) {
    if (!s) return setErr(HS_EINVAL, "null solver");
    uint32_t p;
    int rc;
    if ((rc = poolIndex(s, pool, &p))) return rc;
    double cur;
    if ((rc = readDev(s, s->dc.iCa + p, &cur))) return rc;
    return writeDev(s, s->dc.iCa + p, cur + ica);
}

int hs_push_events(HsSolver* s, const uint32_t* syn, const double* time, const double* weight,
                   uint32_t n) {
    if (!s) return setErr(HS_EINVAL, "null solver");
    if (n == 0) return HS_OK;
    if (!syn || !time || !weight) return setErr(HS_EINVAL, "null argument");
    for (uint32_t i = 0; i < n; ++i) {
        if (syn[i] >= s->P.S) return setErr(HS_EINVAL, "event SynChan index out of range");
        if (std::isnan(time[i])) return setErr(HS_EINVAL, "event time is NaN");
    }
    s->pendSyn.insert(s->pendSyn.end(), syn, syn + n);
    s->pendTime.insert(s->pendTime.end(), time, time + n);
    s->pendW.insert(s->pendW.end(), weight, weight + n);
    return HS_OK;
}

int hs_read_vm(HsSolver* s, double* out, uint32_t n) {
    if (!s || !out) return setErr(HS_EINVAL, "null argument");
    if (n != s->P.hinesOf.size()) return setErr(HS_EINVAL, "n must equal the model's compartment count");
    if (int rc = flushWrites(s)) return rc;
    std::vector<double> v(s->P.N);
    cudaError_t e = cudaMemcpyAsync(v.data(), s->dc.V, v.size() * 8, cudaMemcpyDeviceToHost, stOf(s));
    if (e == cudaSuccess) e = cudaStreamSynchronize(stOf(s));
    if (e != cudaSuccess) return cudaErr(e, "read vm");
    for (uint32_t m = 0; m < n; ++m) out[m] = s->P.hinesOf[m] < 0 ? NAN : v[s->P.hinesOf[m]];
    return HS_OK;
}

int hs_read_ca(HsSolver* s, double* out, uint32_t n) {
    if (!s || !out) return setErr(HS_EINVAL, "null argument");
    if (n != s->P.poolSolverOf.size()) return setErr(HS_EINVAL, "n must equal the model's pool count");
    if (int rc = flushWrites(s)) return rc;
    std::vector<double> v(s->P.P + 1);
    cudaError_t e = cudaMemcpyAsync(v.data(), s->dc.ca, s->P.P * 8, cudaMemcpyDeviceToHost, stOf(s));
    if (e == cudaSuccess) e = cudaStreamSynchronize(stOf(s));
    if (e != cudaSuccess) return cudaErr(e, "read ca");
    for (uint32_t m = 0; m < n; ++m) out[m] = s->P.poolSolverOf[m] < 0 ? NAN : v[s->P.poolSolverOf[m]];
    return HS_OK;
}

int hs_read_dif(HsSolver* s, double* out, uint32_t n) {
    if (!s || (!out && n)) return setErr(HS_EINVAL, "null argument");
    if (n != s->P.nDif) return setErr(HS_EINVAL, "n must equal the model's tick-1 object count");
    if (!n) return HS_OK;
    if (int rc = flushWrites(s)) return rc;
    std::vector<double> st((size_t)kDifState * n);
    cudaError_t e = cudaMemcpyAsync(st.data(), s->dc.difState, st.size() * 8, cudaMemcpyDeviceToHost, stOf(s));
    if (e == cudaSuccess) e = cudaStreamSynchronize(stOf(s));
    if (e != cudaSuccess) return cudaErr(e, "read tick-1 objects");
    for (uint32_t k = 0; k < n; ++k) {
        const int kind = s->P.difKind[k];
        out[k] = kind == HS_DIF_SHELL ? st[k] : kind == HS_DIF_BUFFER ? st[4 * (size_t)n + k] : 0.0;
    }
    return HS_OK;
}

}  // extern "C"

namespace {
// Replaces the solver's recording by `rows` (device recording entries, see
// kRecShift in hs_device.cuh), every target already checked.
int installRecording(HsSolver* s, std::vector<uint32_t>&& rows, uint32_t stride, uint32_t capacity) {
    const uint32_t n = (uint32_t)rows.size();
    cudaStreamSynchronize(stOf(s));
    // From here on the step kernel sees no recording until the new one is
    // complete, so it never writes into a released buffer.
    s->dc.nRec = 0;
    s->dc.recCompt = nullptr;
    s->dc.recBuf = nullptr;
    if (s->recCompt) cudaFree(s->recCompt);
    if (s->recBuf) cudaFree(s->recBuf);
    s->recCompt = nullptr;
    s->recBuf = nullptr;
    s->recHost = std::move(rows);
    // The sample count restarts with the new buffer (reinit sets it again).
    cudaError_t e = cudaMemsetAsync(&s->dc.ctl->nSamples, 0, sizeof(uint32_t), stOf(s));
    if (e != cudaSuccess) return cudaErr(e, "record");
    if (!n) return HS_OK;
    e = cudaMalloc(&s->recCompt, n * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&s->recBuf, (size_t)n * capacity * sizeof(double));
    if (e == cudaSuccess) e = cudaMemsetAsync(s->recBuf, 0, (size_t)n * capacity * sizeof(double), stOf(s));
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->recCompt, s->recHost.data(), n * 4, cudaMemcpyHostToDevice, stOf(s));
    if (e == cudaSuccess) e = cudaStreamSynchronize(stOf(s));
    if (e != cudaSuccess) {
        if (s->recCompt) cudaFree(s->recCompt);
        if (s->recBuf) cudaFree(s->recBuf);
        s->recCompt = nullptr;
        s->recBuf = nullptr;
        s->recHost.clear();
        return cudaErr(e, "record");
    }
    s->dc.nRec = n;
    s->dc.recLd = n;
    s->dc.recStride = stride;
    s->dc.recCap = capacity;
    s->dc.recCompt = s->recCompt;
    s->dc.recBuf = s->recBuf;
    return HS_OK;
}

}  // namespace

extern "C" {

int hs_record(HsSolver* s, const uint32_t* compts, uint32_t n, uint32_t stride, uint32_t capacity) {
    if (!s) return setErr(HS_EINVAL, "null solver");
    if (n && (!compts || stride == 0 || capacity == 0)) return setErr(HS_EINVAL, "bad recording request");
    // Every target is checked before the old recording is released, so a
    // rejected request leaves the previous recording in place.
    std::vector<uint32_t> rows;
    rows.reserve(n);
    for (uint32_t r = 0; r < n; ++r) {
        uint32_t h;
        int rc = comptIndex(s, compts[r], &h);
        if (rc) return rc;
        rows.push_back(h | (kRecVm << kRecShift));
    }
    return installRecording(s, std::move(rows), stride, capacity);
}

int hs_record_values(HsSolver* s, const int* kind, const int* field, const uint32_t* index, uint32_t n,
                     uint32_t stride, uint32_t capacity) {
    if (!s) return setErr(HS_EINVAL, "null solver");
    if (n && (!kind || !field || !index || stride == 0 || capacity == 0))
        return setErr(HS_EINVAL, "bad recording request");
    std::vector<uint32_t> rows;
    rows.reserve(n);
    for (uint32_t r = 0; r < n; ++r) {
        uint32_t i = 0, code;
        int rc;
        if (kind[r] == HS_KIND_COMPT && field[r] == HS_F_VM) {
            rc = comptIndex(s, index[r], &i);
            code = kRecVm;
        } else if (kind[r] == HS_KIND_CHAN && (field[r] == HS_F_IK || field[r] == HS_F_GK)) {
            rc = chanIndex(s, index[r], &i);
            code = field[r] == HS_F_IK ? kRecIk : kRecGk;
        } else if (kind[r] == HS_KIND_POOL && field[r] == HS_F_CA) {
            rc = poolIndex(s, index[r], &i);
            code = kRecCa;
        } else {
            return setErr(HS_EINVAL, "recordable values: compartment Vm, channel Ik or Gk, pool Ca");
        }
        if (rc) return rc;
        if (i >> kRecShift) return setErr(HS_ECAPACITY, "recorded index beyond the recorder's range");
        rows.push_back(i | (code << kRecShift));
    }
    return installRecording(s, std::move(rows), stride, capacity);
}

int hs_read_trace(HsSolver* s, double* out, uint32_t capacity, uint32_t* n_samples) {
    if (!s || !n_samples) return setErr(HS_EINVAL, "null argument");
    if (int rc = flushWrites(s)) return rc;
    DevCtl ctl;
    cudaError_t e = cudaMemcpyAsync(&ctl, s->dc.ctl, sizeof(ctl), cudaMemcpyDeviceToHost, stOf(s));
    if (e == cudaSuccess) e = cudaStreamSynchronize(stOf(s));
    if (e != cudaSuccess) return cudaErr(e, "read trace");
    uint32_t stored = ctl.nSamples < s->dc.recCap ? ctl.nSamples : s->dc.recCap;
    *n_samples = ctl.nSamples;
    if (out && s->dc.nRec) {
        uint32_t k = stored < capacity ? stored : capacity;
        e = cudaMemcpy(out, s->dc.recBuf, (size_t)k * s->dc.nRec * 8, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cudaErr(e, "read trace");
    }
    return HS_OK;
}

int hs_read_spikes(HsSolver* s, uint32_t* gen, double* time, uint32_t capacity, uint32_t* n) {
    if (!s || !n) return setErr(HS_EINVAL, "null argument");
    if (int rc = flushWrites(s)) return rc;
    DevCtl ctl;
    cudaError_t e = cudaMemcpyAsync(&ctl, s->dc.ctl, sizeof(ctl), cudaMemcpyDeviceToHost, stOf(s));
    if (e == cudaSuccess) e = cudaStreamSynchronize(stOf(s));
    if (e != cudaSuccess) return cudaErr(e, "read spikes");
    *n = ctl.nSpikes;
    uint32_t stored = ctl.nSpikes < s->dc.spikeCap ? ctl.nSpikes : s->dc.spikeCap;
    uint32_t k = stored < capacity ? stored : capacity;
    if (k && gen) e = cudaMemcpy(gen, s->dc.spikeGen, k * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && k && time) e = cudaMemcpy(time, s->dc.spikeTime, k * 8, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cudaErr(e, "read spikes");
    if (ctl.nSpikes > s->dc.spikeCap) return setErr(HS_ECAPACITY, "spike buffer overflowed");
    return HS_OK;
}

}  // extern "C"
