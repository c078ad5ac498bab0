// hs_mixed.cu -- mixed-precision batched HSolve step (sm_103a).
//
// A persistent kernel: each CTA owns a list of forests (groups of cells,
// hs_mixed.cuh) packed by size on the host and steps each forest for
// `nsteps` steps before moving on.  Per step, the whole CTA:
//   tick 0    stimulus schedule (a thread per cell)
//   assembly  every node in parallel: FP32 rate lookup and gate update for
//             each channel slot, conductances, the K(Ca) 2-D gate, SynChans;
//             FP64 matrix row into the elimination arrays
//   forward   levels deepest first, a barrier per level: pull the children's
//             eliminated rows, FP64 pivot reciprocal
//   backward  levels root first: VMid = g - f * VMid[parent] (FP64)
//   update    V = 2 VMid - V, Ca pools (FP32)
//   outputs   SpikeGens, trace samples (a thread per cell).
// The update and outputs of a step are done at the start of the next step's
// assembly (and after the last step), which saves a pass over the nodes.
// Reference routines: hsolve/HSolveActive.cpp:45-332, hsolve/HSolvePassive.cpp:
// 246-401 (the same elimination, tree form), biophysics/HHChannel2D.cpp:327-369,
// biophysics/SynChan.cpp:200-224, synapse/SimpleSynHandler.cpp:98-113,
// biophysics/SpikeGen.cpp:202-216.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "hs_mixed.cuh"

namespace hsg {


// Stop step of a cell (none unless the batch set some).
__device__ __forceinline__ unsigned long long stopOf(const MixBatch& b, uint32_t cell) {
    return b.anyStop ? b.stopStep[cell] : ~0ull;
}

// The batch's channel type `tj` (one 16-byte read-only load).
__device__ __forceinline__ ChanType chanType(const MixBatch& b, uint32_t tj) {
    const uint4 v = __ldg(reinterpret_cast<const uint4*>(b.chanTypes + tj));
    ChanType t;
    *reinterpret_cast<uint4*>(&t) = v;
    return t;
}

// Reciprocal of a positive FP64 pivot: the hardware FP64 reciprocal
// estimate (rcp.approx.ftz.f64, relative error about 1e-6 measured over
// 1e-9..1e9) refined by one Newton-Raphson step x <- x + x(1 - d x), which
// squares the error (about 1e-12).
__device__ __forceinline__ double rcpPivot(double d) {
    double x;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(x) : "d"(d));
    const double e = fma(-d, x, 1.0);
    return fma(x, e, x);
}

__device__ __forceinline__ float powi(float x, int p, float pf) {
    switch (p) {
    case 1: return x;
    case 2: return x * x;
    case 3: return x * x * x;
    case 4: { float y = x * x; return y * y; }
    default: return x > 0.f ? __powf(x, pf) : 0.f;
    }
}

struct RowF {
    const float* p;
    float frac;
};

__device__ __forceinline__ RowF rowF(const float* T, uint32_t nCol, uint32_t nRows, float x, float mn,
                                     float mx, float invDx) {
    x = fminf(fmaxf(x, mn), mx);
    float div = (x - mn) * invDx;
    unsigned int i = min((unsigned int)div, nRows - 2);   // rows i and i+1 exist
    RowF r;
    r.frac = div - (float)i;
    r.p = T + (size_t)i * nCol;
    return r;
}

// Exact widening of an FP32 value to FP64 with integer operations (the
// FP32-to-FP64 conversion instruction issues at the FP64 rate on this GPU,
// integer operations at the full rate).  IEEE binary32 -> binary64: sign
// kept, exponent rebiased by 1023 - 127 = 896, fraction shifted left by 29;
// zero and subnormal inputs give a signed zero, Inf/NaN stay Inf/NaN.
__device__ __forceinline__ double widenF(float x) {
    const uint32_t u = __float_as_uint(x);
    const uint32_t e = (u >> 23) & 0xFFu;
    const uint32_t sign = u & 0x80000000u;
    const uint32_t e64 = e == 0xFFu ? 0x7FFu : e + 896u;
    const uint32_t hi = e == 0 ? sign : (sign | (e64 << 20) | ((u >> 3) & 0xFFFFFu));
    const uint32_t lo = e == 0 ? 0u : (u << 29);
    return __hiloint2double((int)hi, (int)lo);
}

// Lerp of the table row pair for column `col` (A at col, B at col + 1).
__device__ __forceinline__ float2 lookupF(const RowF& r, uint32_t nCol, int col) {
    const float* ap = r.p + col;
    const float2 a = __ldg(reinterpret_cast<const float2*>(ap));
    const float2 b = __ldg(reinterpret_cast<const float2*>(ap + nCol));
    return make_float2(fmaf(b.x - a.x, r.frac, a.x), fmaf(b.y - a.y, r.frac, a.y));
}

// A gate state held as the unevaluated sum hi + lo of two FP32 numbers
// (|lo| <= ulp(hi)/2), about 48 significant bits.  Adding an FP32 increment
// uses Knuth's TwoSum (the exact rounding error of hi + d) and Dekker's
// Fast2Sum to renormalise, all on the FP32 pipe: a plain FP32 state would
// lose the small per-step increments of slow gates, and an FP64 add issues
// at 1/64 of the FP32 rate on this GPU, on the pipe the elimination needs.
__device__ __forceinline__ float2 addPair(float2 x, float d) {
    const float s = __fadd_rn(x.x, d);
    const float bv = __fsub_rn(s, x.x);
    const float err = __fadd_rn(__fsub_rn(x.x, __fsub_rn(s, bv)), __fsub_rn(d, bv));
    const float lo = __fadd_rn(x.y, err);
    const float hi = __fadd_rn(s, lo);
    return make_float2(hi, __fsub_rn(lo, __fsub_rn(hi, s)));
}

// New value of a gate with state x over one step, from C1, C2 of its table
// row.  The reference's trapezoidal step (x(2-T) + dt C1)/T with T = 1 + h,
// h = dt/2 C2 (hsolve/HSolveActive.cpp:272-273) is the same number as
// x + (dt C1 - 2 h x)/(1 + h): the increment is computed in FP32 and added
// to the two-float state.  Instantaneous gates: x = C1/C2.
__device__ __forceinline__ float2 gateStep(float2 C, float2 x, float dt, float hdt, bool inst) {
    if (inst) return make_float2(__fdividef(C.x, C.y), 0.f);
    const float h = hdt * C.y;
    return addPair(x, __fdividef(fmaf(-2.0f * h, x.x, dt * C.x), 1.0f + h));
}

__device__ __forceinline__ void interp2dF(const float* T, const float* geom, uint32_t nx, uint32_t ny,
                                          float x, float y, float& A, float& B) {
    x = fminf(fmaxf(x, geom[0]), geom[4]);
    y = fminf(fmaxf(y, geom[1]), geom[5]);
    float xv = (x - geom[0]) * geom[2];
    float yv = (y - geom[1]) * geom[3];
    uint32_t xi = min((uint32_t)xv, nx - 1), yi = min((uint32_t)yv, ny - 1);
    float xF = xv - (float)xi, yF = yv - (float)yi;
    bool endX = xi == nx - 1, endY = yi == ny - 1;
    const float* p00 = T + 2 * ((size_t)xi * ny + yi);
    const float2 z00 = __ldg(reinterpret_cast<const float2*>(p00));
    float2 z10 = make_float2(0.f, 0.f), z01 = z10, z11 = z10;
    if (!endX) z10 = __ldg(reinterpret_cast<const float2*>(p00 + 2 * ny));
    if (!endY) z01 = __ldg(reinterpret_cast<const float2*>(p00 + 2));
    if (!endX && !endY) z11 = __ldg(reinterpret_cast<const float2*>(p00 + 2 * ny + 2));
    float xFyF = xF * yF;
    float w00 = 1.f - xF - yF + xFyF, w10 = xF - xFyF, w01 = yF - xFyF;
    A = z00.x * w00 + z10.x * w10 + z01.x * w01 + z11.x * xFyF;
    B = z00.y * w00 + z10.y * w10 + z01.y * w01 + z11.y * xFyF;
}

// One compartment node of the assembly: first the update left over from the
// previous step (V = 2 VMid - V, then the node's Ca pool; `update`), then
// channels, K(Ca), SynChans and the FP64 matrix row.  Every load that depends
// only on the node index is issued before any arithmetic, so a thread's
// memory round trips per node are: node data, then rate tables and synapse
// state, then (synapses only) event times.
__device__ __forceinline__ void assembleNode(const MixBatch& b, uint32_t n, uint32_t info, bool update,
                                             double vmPrev, unsigned long long step, double& diag, double& rhs) {
    const uint64_t ld = b.ld;
    const float dt = b.dtf, hdt = 0.5f * b.dtf;
    // ---- node data
    double V = b.V[n];
    const uint32_t types = __ldg(b.ctype4 + n);
    const double hs2 = __ldg(b.HS2 + n), cmdt = __ldg(b.CmByDt + n), emrm = __ldg(b.EmByRm + n);
    float gb[kMaxChan];
#pragma unroll
    for (int j = 0; j < kMaxChan; ++j) gb[j] = ((types >> (8 * j)) & 0xFF) != kNoType ? __ldg(b.gbar + (uint64_t)j * ld + n) : 0.f;
    const bool pool = info & kNodePool;
    float ca = 0.f, c0v = 0.f, pg1 = 0.f, pf2 = 0.f, pbas = 0.f, pceil = 0.f, pfloor = 0.f, cgP = 0.f, cgeP = 0.f;
    if (pool) {
        ca = b.poolCa[n];
        if (update) {
            c0v = b.poolC[n];
            pg1 = __ldg(b.poolG1 + n);
            pf2 = __ldg(b.poolF2 + n);
            pbas = __ldg(b.poolBasal + n);
            pceil = __ldg(b.poolCeil + n);
            pfloor = __ldg(b.poolFloor + n);
            cgP = b.caG[n];
            cgeP = b.caGE[n];
        }
    }
    const uint32_t k2 = (info >> 8) & 0xFF;
    float k2x = 0.f, k2g = 0.f;
    if (k2 != kNoType) {
        k2x = b.k2x[n];
        k2g = __ldg(b.k2gbar + n);
    }
    uint32_t s0 = 0, s1 = 0;
    if (info & kNodeSyn) {
        s0 = __ldg(b.syn0 + n);
        s1 = __ldg(b.syn0 + n + 1);
    }
    double inj = 0.0;
    if (info & kNodeInject) inj = b.injVal[__ldg(b.injIdx + n)];
    // ---- the previous step's update
    if (update) {
        const double Vold = V;
        V = fma(2.0, vmPrev, -Vold);
        b.V[n] = V;
        if (pool) {
            const float vca = (float)(b.caAdvance == 1 ? vmPrev : fma(2.0, vmPrev, -V));
            const float act = fmaf(-cgP, vca, cgeP);
            // c f1 + f2 act with f1 = 1 - g1 (g1 = 1 - f1 from FP64)
            float c = fmaf(-pg1, c0v, c0v) + pf2 * act;
            float cav = pbas + c;
            if (pceil > 0.f && cav > pceil) { cav = pceil; c = cav - pbas; }
            if (cav < pfloor) { cav = pfloor; c = cav - pbas; }
            b.poolC[n] = c;
            b.poolCa[n] = cav;
            ca = cav;
        }
    }
    // ---- HHChannels: trapezoidal gates on the V (or Ca) table rows
    const float v = (float)V;
    const RowF vr = rowF(b.vTab, b.vCol, b.vRows, v, b.vMin, b.vMax, b.vInvDx);
    float G = 0.f, GE = 0.f, cg = 0.f, cge = 0.f;
#pragma unroll
    for (int j = 0; j < kMaxChan; ++j) {
        const uint32_t tj = (types >> (8 * j)) & 0xFF;
        if (tj == kNoType) continue;
        const ChanType t = chanType(b, tj);
        float2* st = b.state + (uint64_t)(3 * j) * ld + n;
        float frac = 1.f;
        if (t.xp) {
            const float2 x = gateStep(lookupF(vr, b.vCol, t.colX), st[0], dt, hdt, t.instant & 1);
            st[0] = x;
            frac *= powi(x.x, t.xp, t.xp < 0 ? __ldg(&b.chanPow[tj].x) : 0.f);
        }
        if (t.yp) {
            const float2 y = gateStep(lookupF(vr, b.vCol, t.colY), st[ld], dt, hdt, t.instant & 2);
            st[ld] = y;
            frac *= powi(y.x, t.yp, t.yp < 0 ? __ldg(&b.chanPow[tj].y) : 0.f);
        }
        if (t.zp) {
            float2 C;
            if (t.zCa) C = lookupF(rowF(b.caTab, b.caCol, b.caRows, ca, b.caMin, b.caMax, b.caInvDx), b.caCol, t.colZ);
            else C = lookupF(vr, b.vCol, t.colZ);
            const float2 z = gateStep(C, st[2 * ld], dt, hdt, t.instant & 4);
            st[2 * ld] = z;
            frac *= powi(z.x, t.zp, t.zp < 0 ? __ldg(&b.chanPow[tj].z) : 0.f);
        }
        const float gk = gb[j] * frac;
        G += gk;
        GE = fmaf(gk, t.ek, GE);
        if (t.caTarget) {
            cg += gk;
            cge = fmaf(gk, t.ek, cge);
        }
    }
    if (pool) {
        b.caG[n] = cg;
        b.caGE[n] = cge;
    }
    // ---- HHChannel2D (K(Ca)) on this step's Vm and Ca
    if (k2 != kNoType) {
        const C2dType& t = b.c2dTypes[k2];
        const float x = t.dep0 == 0 ? v : t.dep0 == 1 ? ca : 0.f;
        const float y = t.dep1 == 0 ? v : t.dep1 == 1 ? ca : 0.f;
        float A, B;
        interp2dF(b.g2d + b.g2dOff[t.gate], b.g2dGeom + 6 * t.gate, b.g2dN[2 * t.gate], b.g2dN[2 * t.gate + 1], x,
                  y, A, B);
        float X = k2x;
        if (t.instant & 1) X = __fdividef(A, B);
        else if (B > 1.0e-10f) {
            // HHChannelBase::integrate, X e + (A/B)(1 - e) with e = exp(-B dt),
            // as X + (A/B - X)(1 - e), 1 - e = -expm1(-B dt) (no cancellation)
            const float em = -expm1f(-B * dt);
            X = fmaf(__fdividef(A, B) - X, em, X);
        } else X = fmaf(A, dt, X);
        b.k2x[n] = X;
        const float gk = k2g * powi(X, t.xp, t.xpf);
        G += gk;
        GE = fmaf(gk, t.ek, GE);
    }
    // ---- SynChans: conductances of this step, advanced beforehand (synapseStep)
    for (uint32_t k = s0; k < s1; ++k) {
        const float2 g = b.synGk[k];
        G += g.x;
        GE += g.y;
    }
    diag = hs2 + widenF(G);
    rhs = fma(V, cmdt, emrm) + widenF(GE) + inj;
}

// SynChan k over step `step`: the events delivered (SimpleSynHandler, weight
// / dt each), the dual exponential X, Y, and the conductance Gk and Gk Ek
// the assembly of that step adds.  Needs no Vm, so it runs ahead of the
// assembly (see stepForest).
__device__ __forceinline__ void synapseStep(const MixBatch& b, uint32_t k, unsigned long long step) {
    if (step >= stopOf(b, __ldg(b.synCell + k))) return;
    const SynType& t = b.synTypes[__ldg(b.synType + k)];
    uint32_t e = b.evCur[k];
    const uint32_t end = __ldg(b.evEnd + k);
    const float sx = b.synX[k], sy = b.synY[k], nm = __ldg(b.synNorm + k);
    float act = 0.f;
    while (e < end && __ldg(b.evStep + e) <= step) act += __ldg(b.evAct + e++);
    b.evCur[k] = e;
    const float X = fmaf(act, t.xc1, sx * t.xc2);
    const float Y = fmaf(X, t.yc1, sy * t.yc2);
    b.synX[k] = X;
    b.synY[k] = Y;
    const float gk = Y * nm;
    b.synGk[k] = make_float2(gk, gk * t.ek);
}

// Elimination arrays of a forest: pivots/couplings D, right-hand sides R,
// off-diagonals OFF, topology TOPO and PAR (forest-local indices).
struct Elim {
    double *D, *R;
    const double* OFF;
    const uint32_t* TOPO;
    const uint16_t* PAR;
};

// Per-cell work of tick 0 (stimulus schedule) for the forest's cells.
__device__ __forceinline__ void forestStimulus(const MixBatch& b, const MixForest& F, unsigned long long step) {
    for (uint32_t k = threadIdx.x; k < F.nCells; k += blockDim.x) {
        const uint32_t cell = b.forestCells[F.cell0 + k];
        const MixCellRange cr = b.cells[cell];
        if (!cr.nStim || step >= stopOf(b, cell)) continue;
        uint32_t cur = b.stimCur[cell];
        while (cur < cr.nStim && b.stimStep[cr.stim0 + cur] <= step) {
            b.injVal[cr.inj0 + b.stimEntry[cr.stim0 + cur]] = b.stimValue[cr.stim0 + cur];
            ++cur;
        }
        b.stimCur[cell] = cur;
    }
}

// SpikeGens (SpikeGen::process with the solver's V and currTime = dt (step+1))
// and trace samples, one thread per cell.
__device__ __forceinline__ void forestOutputs(const MixBatch& b, const MixForest& F, unsigned long long step,
                                              uint32_t t0, uint32_t nt) {
    const double currTime = b.dt * (double)(step + 1);
    const bool sample = ((step + 1) % b.recStride) == 0;
    for (uint32_t k = t0; k < F.nCells; k += nt) {
        const uint32_t cell = b.forestCells[F.cell0 + k];
        if (step >= stopOf(b, cell)) continue;
        const MixCellRange cr = b.cells[cell];
        for (uint32_t g = cr.sg0; g < cr.sg0 + cr.nSg; ++g) {
            const double Vs = b.V[b.sgNode[g]];
            if (Vs > (double)b.sgThresh[g]) {
                if ((float)(currTime + b.dt / 2.0) >= b.sgLast[g] + b.sgRefract[g] && !(b.sgEdge[g] && b.sgFired[g])) {
                    const uint32_t spk = b.spikeCount[cell];
                    if (spk < b.spikeCap) {
                        b.spikeGen[(size_t)cell * b.spikeCap + spk] = g - cr.sg0;
                        b.spikeTime[(size_t)cell * b.spikeCap + spk] = (float)currTime;
                    }
                    b.spikeCount[cell] = spk + 1;
                    b.sgLast[g] = (float)currTime;
                    b.sgFired[g] = 1;
                }
            } else {
                b.sgFired[g] = 0;
            }
        }
        if (cr.nRec && sample) {
            const uint64_t smp = (step + 1) / b.recStride;
            if (smp < b.recCap)
                for (uint32_t r = cr.rec0; r < cr.rec0 + cr.nRec; ++r)
                    b.recBuf[smp * b.recLd + r] = b.V[b.recNode[r]];
        }
    }
}

// Bulk prefetch into L2 (cp.async.bulk.prefetch) of forest nodes
// [first, first + count) of per-node array `k`, clamped to the array and
// aligned to 16 bytes; called by one thread per array.
__device__ __forceinline__ void prefetchNodes(const MixBatch& b, uint32_t k, uint64_t first, uint32_t count) {
    const PrefetchArr a = b.pf[k];
    const uint64_t total = (uint64_t)a.n * a.elem / 16 * 16;
    uint64_t lo = first * a.elem / 16 * 16;
    uint64_t hi = ((first + count) * a.elem + 15) / 16 * 16;
    if (hi > total) hi = total;
    if (lo >= hi) return;
    const char* p = static_cast<const char*>(a.base) + lo;
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"((uint32_t)(hi - lo)) : "memory");
}

// V = 2 VMid - V, then the node's Ca pool: the end of a step of one node.
__device__ __forceinline__ void updateNode(const MixBatch& b, uint32_t n, uint32_t info, double vm) {
    const double Vnew = fma(2.0, vm, -b.V[n]);
    b.V[n] = Vnew;
    if (info & kNodePool) {
        const float vca = (float)(b.caAdvance == 1 ? vm : fma(2.0, vm, -Vnew));
        const float act = fmaf(-b.caG[n], vca, b.caGE[n]);
        const float c0v = b.poolC[n];
        float c = fmaf(-b.poolG1[n], c0v, c0v) + b.poolF2[n] * act;
        float cav = b.poolBasal[n] + c;
        if (b.poolCeil[n] > 0.f && cav > b.poolCeil[n]) { cav = b.poolCeil[n]; c = cav - b.poolBasal[n]; }
        if (cav < b.poolFloor[n]) { cav = b.poolFloor[n]; c = cav - b.poolBasal[n]; }
        b.poolC[n] = c;
        b.poolCa[n] = cav;
    }
}

// After a forest's last step (`step` = steps done): that step's update and
// outputs, the per-cell step counts and the forest's counter.
__device__ void finishForest(const MixBatch& b, const MixForest& F, uint32_t f, const Elim& E,
                             unsigned long long step) {
    const uint32_t tid = threadIdx.x, nth = blockDim.x;
    for (uint32_t i = tid; i < F.nNodes; i += nth) {
        const uint32_t n = F.node0 + i;
        const uint32_t info = __ldg(b.nodeInfo + n);
        if (info & kNodeCenter) continue;
        if (step - 1 < stopOf(b, __ldg(b.cellOf + n))) updateNode(b, n, info, E.R[i]);
    }
    __syncthreads();
    forestOutputs(b, F, step - 1, tid, nth);
    for (uint32_t k = tid; k < F.nCells; k += nth) {
        const uint32_t cell = b.forestCells[F.cell0 + k];
        const unsigned long long stop = stopOf(b, cell);
        b.stepCount[cell] = step < stop ? step : stop;
    }
    if (tid == 0) b.forestStep[f] = step;
    __syncthreads();
}

// `nsteps` steps of one forest by the whole CTA.  The V/Ca update and the
// outputs (SpikeGens, trace samples) of a step run at the start of the next
// step's assembly, and after the last step.  A cell whose stop step is
// reached stays as it is: its nodes get a neutral row (pivot 1, rhs 0) so
// that the elimination of the forest goes on around them.
__device__ void stepForest(const MixBatch& b, const MixForest& F, uint32_t f, const Elim& E, const uint32_t* lp,
                           uint32_t nsteps) {
    const uint32_t tid = threadIdx.x, nth = blockDim.x;
    if (nsteps == 0) return;
    unsigned long long step = b.forestStep[f];
    // SynChans of the forest: [k0, k1).  Those of step 0 of the launch are
    // advanced here; those of every later step by the threads that a level of
    // the previous step's elimination leaves idle (whole idle warps take the
    // next synapses in order), the rest after that elimination.
    const uint32_t k0 = __ldg(b.syn0 + F.node0), k1 = __ldg(b.syn0 + F.node0 + F.nNodes);
    for (uint32_t k = k0 + tid; k < k1; k += nth) synapseStep(b, k, step);
    for (uint32_t s = 0; s < nsteps; ++s, ++step) {
        if (tid < b.nPf) prefetchNodes(b, tid, F.node0, nth);
        forestStimulus(b, F, step);
        __syncthreads();
        // assembly: every node's FP64 row (junction nodes: their diagonal);
        // the next chunk of nth nodes is prefetched into L2 meanwhile
        for (uint32_t i = tid; i < F.nNodes; i += nth) {
            if (tid < b.nPf && i + nth - tid < F.nNodes) prefetchNodes(b, tid, F.node0 + i + nth - tid, nth);
            const uint32_t n = F.node0 + i;
            const uint32_t info = __ldg(b.nodeInfo + n);
            const unsigned long long stop = b.anyStop ? b.stopStep[__ldg(b.cellOf + n)] : ~0ull;
            const bool live = step < stop;                  // this step advances the cell
            const bool pending = s > 0 && step - 1 < stop;  // the previous step's update
            double d = 1.0, r = 0.0;
            if (info & kNodeCenter) {
                if (live) d = __ldg(b.HS2 + n);
            } else if (live) {
                assembleNode(b, n, info, pending, pending ? E.R[i] : 0.0, step, d, r);
            } else if (pending) {
                updateNode(b, n, info, E.R[i]);
            }
            E.D[i] = d;
            E.R[i] = r;
        }
        __syncthreads();
        if (s > 0) forestOutputs(b, F, step - 1, tid, nth);
        // forward elimination, deepest level first: pull the children's
        // eliminated rows (diag -= off_c * f_c, rhs -= off_c * g_c), then keep
        // g = rhs/pivot in R and f = off/pivot in D
        const bool ahead = s + 1 < nsteps;     // advance the next step's synapses
        uint32_t kNext = k0;
        for (int L = (int)F.nLevels - 1; L >= 0; --L) {
            const uint32_t e = lp[L + 1];
            if (ahead && kNext < k1) {
                const uint32_t busy = (e - lp[L] + 31) & ~31u;
                if (busy < nth) {
                    if (tid >= busy && kNext + (tid - busy) < k1) synapseStep(b, kNext + (tid - busy), step + 1);
                    kNext += nth - busy;
                }
            }
            for (uint32_t i = lp[L] + tid; i < e; i += nth) {
                const uint32_t t = E.TOPO[i];
                const uint32_t c0 = t & 0xFFFF, c1 = c0 + ((t >> 16) & 0xFF);
                double d = E.D[i], r = E.R[i];
                for (uint32_t c = c0; c < c1; ++c) {
                    const double oc = E.OFF[c];
                    d = fma(-oc, E.D[c], d);
                    r = fma(-oc, E.R[c], r);
                }
                const double iv = rcpPivot(d);
                E.R[i] = r * iv;
                E.D[i] = E.OFF[i] * iv;
            }
            __syncthreads();
        }
        // back substitution, root level first: VMid = g - f * VMid[parent]
        for (uint32_t L = 0; L < F.nLevels; ++L) {
            const uint32_t e = lp[L + 1];
            for (uint32_t i = lp[L] + tid; i < e; i += nth) {
                const uint32_t p = E.PAR[i];
                double vm = E.R[i];
                if (p != kNoParent) vm = fma(-E.D[i], E.R[p], vm);
                E.R[i] = vm;
            }
            __syncthreads();
        }
        if (ahead)
            for (uint32_t k = kNext + tid; k < k1; k += nth) synapseStep(b, k, step + 1);
    }
    finishForest(b, F, f, E, step);
}

// Named barrier over `count` threads (a multiple of 32).
__device__ __forceinline__ void groupSync(uint32_t id, uint32_t count) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}

// Bounded wait of an eliminator for a level's assembly: at most
// b.waitRounds rounds of ~128 ns (default 2^24, far longer than any
// assembly), so that a lost update ends the kernel with an error instead of
// a hang.  A thread that gave up once, or that sees the batch's error flag
// set by another CTA, waits no more in this launch: the launch then ends
// after at most one bounded wait per eliminator thread, and its results are
// marked invalid (hs_batch_sync returns HS_ETIMEOUT).
__device__ __forceinline__ bool waitLevel(const MixBatch& b, const uint32_t* done, uint32_t need, bool& gaveUp) {
    if (gaveUp) return false;
    uint32_t rounds = 0;
    while (*(volatile const uint32_t*)done < need) {
        ++rounds;
        if (rounds > b.waitRounds || ((rounds & 1023u) == 0 && *(volatile const uint32_t*)b.err)) {
            atomicExch(b.err, 1u);
            gaveUp = true;
            return false;
        }
        __nanosleep(128);
    }
    return true;
}

// The same steps as stepForest with the CTA split into two groups.  The
// first `elimWarps` warps eliminate; the others assemble nodes deepest level
// first and count the finished nodes of each level in `done` (shared
// memory).  The eliminators start a level of the forward elimination as soon
// as its count is complete, so the elimination of the deep levels overlaps
// the assembly of the shallow ones; meanwhile the assemblers emit the
// previous step's outputs and advance the next step's SynChans.  Then the
// whole CTA substitutes back.  Forests of at most 255 levels (the level of a node is kept in
// the top byte of its topology word).
__device__ void stepForestWS(const MixBatch& b, const MixForest& F, uint32_t f, const Elim& E, const uint32_t* lp,
                             uint32_t* done, uint32_t elimWarps, uint32_t nsteps) {
    const uint32_t tid = threadIdx.x, nth = blockDim.x;
    if (nsteps == 0) return;
    const uint32_t nE = 32 * elimWarps, nA = nth - nE;
    const bool elim = tid < nE;
    const uint32_t atid = tid - nE;
    unsigned long long step = b.forestStep[f];
    const uint32_t k0 = __ldg(b.syn0 + F.node0), k1 = __ldg(b.syn0 + F.node0 + F.nNodes);
    for (uint32_t k = k0 + tid; k < k1; k += nth) synapseStep(b, k, step);
    bool gaveUp = false;
    for (uint32_t s = 0; s < nsteps; ++s, ++step) {
        for (uint32_t L = tid; L < F.nLevels; L += nth) done[L] = 0;
        forestStimulus(b, F, step);
        __syncthreads();
        if (elim) {
            // forward elimination, each level once the assemblers finished it
            for (int L = (int)F.nLevels - 1; L >= 0; --L) {
                const uint32_t b0 = lp[L], e = lp[L + 1];
                waitLevel(b, &done[L], e - b0, gaveUp);
                __threadfence_block();
                if (2 * (e - b0) <= nE) {
                    // a narrow level: two lanes per node, the even one on the
                    // pivot (D), the odd one on the right-hand side (R), so
                    // that each child costs one FP64 warp instruction instead
                    // of two (the FP64 cost is per warp instruction)
                    const uint32_t i = b0 + (tid >> 1);
                    const bool rl = tid & 1u;
                    const bool on = i < e;
                    const uint32_t t = on ? E.TOPO[i] : 0u;
                    const uint32_t c0 = t & 0xFFFF, c1 = c0 + ((t >> 16) & 0xFF);
                    double* const A = rl ? E.R : E.D;
                    double x = on ? A[i] : 1.0;
                    for (uint32_t c = c0; c < c1; ++c) x = fma(-E.OFF[c], A[c], x);
                    const double ivd = rcpPivot(x);
                    const double iv = __shfl_sync(0xFFFFFFFFu, ivd, (tid & 31u) & ~1u);
                    const double y = (rl ? x : (on ? E.OFF[i] : 0.0)) * iv;
                    if (on) A[i] = y;
                } else {
                    for (uint32_t i = b0 + tid; i < e; i += nE) {
                        const uint32_t t = E.TOPO[i];
                        const uint32_t c0 = t & 0xFFFF, c1 = c0 + ((t >> 16) & 0xFF);
                        double d = E.D[i], r = E.R[i];
                        for (uint32_t c = c0; c < c1; ++c) {
                            const double oc = E.OFF[c];
                            d = fma(-oc, E.D[c], d);
                            r = fma(-oc, E.R[c], r);
                        }
                        const double iv = rcpPivot(d);
                        E.R[i] = r * iv;
                        E.D[i] = E.OFF[i] * iv;
                    }
                }
                groupSync(1, nE);
            }
        } else {
            // assembly, deepest level first (the highest node indices); each
            // node's info word is loaded one node ahead, which takes the
            // first of the node's dependent memory round trips off its chain
            uint32_t infoNext = atid < F.nNodes ? __ldg(b.nodeInfo + F.node0 + F.nNodes - 1 - atid) : 0u;
            for (uint32_t j = atid; j < F.nNodes; j += nA) {
                const uint32_t i = F.nNodes - 1 - j;
                if (atid < b.nPf && j + nA - atid < F.nNodes) {
                    const uint32_t hi = F.nNodes - (j + nA - atid);     // next chunk: [hi - nA, hi)
                    prefetchNodes(b, atid, F.node0 + (hi > nA ? hi - nA : 0), hi > nA ? nA : hi);
                }
                const uint32_t n = F.node0 + i;
                const uint32_t info = infoNext;
                if (j + nA < F.nNodes) infoNext = __ldg(b.nodeInfo + F.node0 + F.nNodes - 1 - (j + nA));
                const unsigned long long stop = b.anyStop ? b.stopStep[__ldg(b.cellOf + n)] : ~0ull;
                const bool live = step < stop;
                const bool pending = s > 0 && step - 1 < stop;
                double d = 1.0, r = 0.0;
                if (info & kNodeCenter) {
                    if (live) d = __ldg(b.HS2 + n);
                } else if (live) {
                    assembleNode(b, n, info, pending, pending ? E.R[i] : 0.0, step, d, r);
                } else if (pending) {
                    updateNode(b, n, info, E.R[i]);
                }
                E.D[i] = d;
                E.R[i] = r;
                __threadfence_block();
                atomicAdd(&done[E.TOPO[i] >> 24], 1u);
            }
            groupSync(2, nA);
            if (s > 0) forestOutputs(b, F, step - 1, atid, nA);
            if (s + 1 < nsteps)
                for (uint32_t k = k0 + atid; k < k1; k += nA) synapseStep(b, k, step + 1);
        }
        __syncthreads();
        // back substitution by the whole CTA
        if (F.shared) {
            for (uint32_t L = 0; L < F.nLevels; ++L) {
                const uint32_t e = lp[L + 1];
                for (uint32_t i = lp[L] + tid; i < e; i += nth) {
                    const uint32_t p = E.PAR[i];
                    double vm = E.R[i];
                    if (p != kNoParent) vm = fma(-E.D[i], E.R[p], vm);
                    E.R[i] = vm;
                }
                __syncthreads();
            }
        } else {
            // in global memory: a thread's first node of the next level has
            // its parent index, coupling and right-hand side (none of which
            // this level changes) loaded before the barrier, leaving one
            // dependent load (the parent's value) per level
            uint32_t nb = lp[0] + tid, ne = lp[1], pn = 0;
            double dn = 0.0, rn = 0.0;
            if (nb < ne) {
                pn = E.PAR[nb];
                dn = E.D[nb];
                rn = E.R[nb];
            }
            for (uint32_t L = 0; L < F.nLevels; ++L) {
                const uint32_t i0 = nb, e = ne, p0 = pn;
                const double d0 = dn, r0 = rn;
                if (L + 1 < F.nLevels) {
                    nb = lp[L + 1] + tid;
                    ne = lp[L + 2];
                    if (nb < ne) {
                        pn = E.PAR[nb];
                        dn = E.D[nb];
                        rn = E.R[nb];
                    }
                }
                if (i0 < e) E.R[i0] = p0 != kNoParent ? fma(-d0, E.R[p0], r0) : r0;
                for (uint32_t i = i0 + nth; i < e; i += nth) {
                    const uint32_t p = E.PAR[i];
                    double vm = E.R[i];
                    if (p != kNoParent) vm = fma(-E.D[i], E.R[p], vm);
                    E.R[i] = vm;
                }
                __syncthreads();
            }
        }
    }
    finishForest(b, F, f, E, step);
}

// One CTA steps its forests one after the other, each for `nsteps` steps.
// Dynamic shared memory: kSmemLevels level offsets, then for shared forests
// the elimination arrays of `cap` nodes: D, R, OFF (8 B each), TOPO (4 B),
// PAR (2 B).
// kStops: the batch has stop steps (b.anyStop); the batches without (the
// throughput case) get an instantiation without the forest check, whose
// registers are allocated as if it did not exist.
template <bool kStops>
__global__ void __launch_bounds__(1024, 1) hsForestStepMixed(MixBatch b, const uint32_t* __restrict__ ctaPtr,
                                                             const uint32_t* __restrict__ ctaForests, uint32_t cap,
                                                             uint32_t elimWarps, uint32_t nsteps) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t* sLp = reinterpret_cast<uint32_t*>(smem);
    uint32_t* sDone = sLp + kSmemLevels;
    double* sD = reinterpret_cast<double*>(smem + (kSmemLevels + kWsLevels) * 4);
    for (uint32_t k = ctaPtr[blockIdx.x]; k < ctaPtr[blockIdx.x + 1]; ++k) {
        const MixForest F = b.forests[ctaForests[k]];
        if (kStops && b.forestStep[ctaForests[k]] >= b.forestStop[ctaForests[k]]) {
            // every cell of the forest has reached its stop step: stepping it
            // would change nothing (stopped cells keep their state, outputs
            // and step counts), so its steps are only counted and the CTA
            // can return and free its SM for other batches
            __syncthreads();
            if (threadIdx.x == 0) b.forestStep[ctaForests[k]] += nsteps;
            continue;
        }
        const uint32_t* lp = b.levelPtr + F.level0;
        if (F.nLevels < kSmemLevels) {
            for (uint32_t i = threadIdx.x; i <= F.nLevels; i += blockDim.x) sLp[i] = lp[i];
            lp = sLp;
        }
        Elim E;
        if (F.shared) {
            double* sR = sD + cap;
            double* sOff = sR + cap;
            uint32_t* sTopo = reinterpret_cast<uint32_t*>(sOff + cap);
            uint16_t* sPar = reinterpret_cast<uint16_t*>(sTopo + cap);
            for (uint32_t i = threadIdx.x; i < F.nNodes; i += blockDim.x) {
                sOff[i] = b.off[F.node0 + i];
                sTopo[i] = b.topo[F.node0 + i];
                sPar[i] = b.par[F.node0 + i];
            }
            E.D = sD;
            E.R = sR;
            E.OFF = sOff;
            E.TOPO = sTopo;
            E.PAR = sPar;
        } else {
            E.D = b.elimD + F.node0;
            E.R = b.elimR + F.node0;
            E.OFF = b.off + F.node0;
            E.TOPO = b.topo + F.node0;
            E.PAR = b.par + F.node0;
        }
        __syncthreads();
        // a forest eliminated in global memory (a cell too large for shared
        // memory, as serving requests can be) has wide levels of slow loads:
        // twice the eliminator warps (measured on a 10,000-compartment cell:
        // 184 -> 159 us per step).  Only in the instantiation for batches
        // with stop steps, so that the throughput kernel's registers stay
        // as they are.
        const uint32_t ew = kStops && !F.shared ? min(2 * elimWarps, 16u) : elimWarps;
        if (ew && F.nLevels <= kWsLevels - 1 && F.nLevels < kSmemLevels && blockDim.x > 32 * ew)
            stepForestWS(b, F, ctaForests[k], E, lp, sDone, ew, nsteps);
        else
            stepForest(b, F, ctaForests[k], E, lp, nsteps);
    }
}

// Reinit, per node: V = initVm, gates at their steady state, Ca = CaBasal,
// synapses, K(Ca) X.
__global__ void hsReinitNodesMixed(MixBatch b, uint32_t nNodes, const double* __restrict__ initVm,
                                   const float* __restrict__ k2x0, const uint32_t* __restrict__ evStart) {
    const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nNodes) return;
    const uint64_t ld = b.ld;
    const uint32_t info = b.nodeInfo[n];
    b.V[n] = initVm[n];
    if (info & kNodeCenter) return;
    if (info & kNodePool) {
        b.poolC[n] = 0.f;
        b.poolCa[n] = b.poolBasal[n];
    }
    const float ca = (info & kNodePool) ? b.poolCa[n] : 0.f;
    RowF vr = rowF(b.vTab, b.vCol, b.vRows, (float)initVm[n], b.vMin, b.vMax, b.vInvDx);
    const uint32_t types = b.ctype4[n];
    for (int j = 0; j < kMaxChan; ++j) {
        const uint32_t tj = (types >> (8 * j)) & 0xFF;
        if (tj == kNoType) break;
        const ChanType t = chanType(b, tj);
        float2* st = b.state + (uint64_t)(3 * j) * ld + n;
        const float2 z0 = make_float2(0.f, 0.f);
        if (t.xp) st[0] = gateStep(lookupF(vr, b.vCol, t.colX), z0, 0.f, 0.f, true);
        if (t.yp) st[ld] = gateStep(lookupF(vr, b.vCol, t.colY), z0, 0.f, 0.f, true);
        if (t.zp) {
            if (t.zCa)
                st[2 * ld] = gateStep(lookupF(rowF(b.caTab, b.caCol, b.caRows, ca, b.caMin, b.caMax, b.caInvDx),
                                              b.caCol, t.colZ), z0, 0.f, 0.f, true);
            else
                st[2 * ld] = gateStep(lookupF(vr, b.vCol, t.colZ), z0, 0.f, 0.f, true);
        }
    }
    if (((info >> 8) & 0xFF) != kNoType) b.k2x[n] = k2x0[n];
    if (info & kNodeSyn)
        for (uint32_t k = b.syn0[n]; k < b.syn0[n + 1]; ++k) {
            b.synX[k] = 0.f;
            b.synY[k] = 0.f;
            b.evCur[k] = evStart[k];
        }
}

// Reinit, per cell: SpikeGens, counters, trace sample 0 (after the nodes).
__global__ void hsReinitCellsMixed(MixBatch b) {
    const uint32_t cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= b.nCells) return;
    const MixCellRange cr = b.cells[cell];
    for (uint32_t g = cr.sg0; g < cr.sg0 + cr.nSg; ++g) {
        b.sgLast[g] = -b.sgRefract[g];
        b.sgFired[g] = 0;
    }
    if (cell < b.nForests) b.forestStep[cell] = 0;
    b.stepCount[cell] = 0;
    b.stimCur[cell] = 0;
    b.spikeCount[cell] = 0;
    for (uint32_t r = cr.rec0; r < cr.rec0 + cr.nRec; ++r) b.recBuf[r] = b.V[b.recNode[r]];
}

// Scatter of host-supplied inject values to their solver slots.
__global__ void hsScatterInject(double* const* __restrict__ addr, uint8_t* const* __restrict__ flag,
                                const double* __restrict__ val, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    *addr[i] = val[i];
    if (flag[i]) *flag[i] = 1;
}

__global__ void hsScatterValues(const ValueWrite* __restrict__ w, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const ValueWrite x = w[i];
    if (x.f32) *static_cast<float*>(x.addr) = (float)x.value;
    else *static_cast<double*>(x.addr) = x.value;
}

cudaError_t launchScatterValues(const ValueWrite* w, uint32_t n, cudaStream_t st) {
    if (!n) return cudaSuccess;
    hsScatterValues<<<(n + 255) / 256, 256, 0, st>>>(w, n);
    return cudaGetLastError();
}

cudaError_t launchScatterInject(double* const* addr, uint8_t* const* flag, const double* val, uint32_t n,
                                cudaStream_t st) {
    if (!n) return cudaSuccess;
    hsScatterInject<<<(n + 255) / 256, 256, 0, st>>>(addr, flag, val, n);
    return cudaGetLastError();
}

// ---- several SMs per forest: a thread-block cluster -------------------------------
// For latency: the forests of one cluster of kC CTAs are stepped by all of
// them together.  A forest's pivots/couplings D and right-hand sides R live
// in rank 0's shared memory (16 B a node; OFF, TOPO and PAR stay in global
// memory); every CTA assembles (rank 0's first `elimWarps` warps excepted),
// writing each node's row into rank 0's D and R through distributed shared
// memory and adding the per-level completion counts there.  Rank 0's
// eliminator warps walk the levels as in stepForestWS, then rank 0 alone
// substitutes back.  The CTAs of the cluster meet at bounded barriers
// (clusterMeet) twice per step: after assembly and elimination, and after the
// back substitution (by when rank 0 has also reset the level counters and
// applied the next step's stimulus).  The arithmetic of every node is
// that of the one-CTA step, so results are bit-identical.

// This CTA's writes (global and shared) made visible at cluster scope.
__device__ __forceinline__ void fenceCluster() { asm volatile("fence.acq_rel.cluster;" ::: "memory"); }

// A bounded barrier of the kC CTAs of a cluster on a counter in rank 0's
// shared memory (`bar`, a distributed shared memory address): each CTA adds
// 1 and waits for the count of this meeting, `gen` x kC.  Every wait is
// bounded by b.waitRounds sleeps; after a timeout, or once the batch's error
// flag is set, a CTA waits no more in this launch (the launch then ends with
// its results marked invalid, as with waitLevel).
__device__ __forceinline__ void clusterMeet(const MixBatch& b, uint32_t* bar, uint32_t& gen, uint32_t kC,
                                            bool& gaveUp) {
    __syncthreads();
    ++gen;
    if (threadIdx.x == 0) {
        fenceCluster();
        atomicAdd(bar, 1u);
        uint32_t rounds = 0;
        while (!gaveUp && *(volatile const uint32_t*)bar < gen * kC) {
            ++rounds;
            if (rounds > b.waitRounds || ((rounds & 1023u) == 0 && *(volatile const uint32_t*)b.err)) {
                atomicExch(b.err, 1u);
                gaveUp = true;
                break;
            }
            __nanosleep(64);
        }
        fenceCluster();
    }
    __syncthreads();
}

// `nsteps` steps of forest F by the cluster.  E.D and E.R point into rank
// 0's shared memory (its own, or through distributed shared memory).
__device__ void stepForestCluster(const MixBatch& b, const MixForest& F, uint32_t f, const Elim& E,
                                  const uint32_t* lp, uint32_t* done, uint32_t* doneR0, uint32_t* barR0,
                                  uint32_t& gen, uint32_t rank, uint32_t kC, uint32_t elimWarps, uint32_t nsteps,
                                  bool& gaveUp) {
    const uint32_t tid = threadIdx.x, nth = blockDim.x;
    const uint32_t nE = rank == 0 ? 32 * elimWarps : 0;
    const bool elim = tid < nE;
    const uint32_t nAL = nth - 32 * elimWarps;              // assemblers of rank 0
    const uint32_t ga = rank == 0 ? tid - nE : nAL + (rank - 1) * nth + tid;
    const uint32_t T = nAL + (kC - 1) * nth;                // assemblers of the cluster
    const uint32_t gt = rank * nth + tid, GT = kC * nth;     // every thread of the cluster
    unsigned long long step = b.forestStep[f];
    const uint32_t k0 = __ldg(b.syn0 + F.node0), k1 = __ldg(b.syn0 + F.node0 + F.nNodes);
    for (uint32_t k = k0 + gt; k < k1; k += GT) synapseStep(b, k, step);
    bool waitGaveUp = false;
    // each step's level counters and stimulus are set before the meeting
    // that ends the step before it (here, for the first step)
    if (rank == 0) {
        for (uint32_t L = tid; L < F.nLevels; L += nth) done[L] = 0;
        forestStimulus(b, F, step);
    }
    clusterMeet(b, barR0, gen, kC, gaveUp);
    for (uint32_t s = 0; s < nsteps; ++s, ++step) {
        if (elim) {
            for (int L = (int)F.nLevels - 1; L >= 0; --L) {
                const uint32_t b0 = lp[L], e = lp[L + 1];
                waitLevel(b, &done[L], e - b0, waitGaveUp);
                fenceCluster();
                if (2 * (e - b0) <= nE) {
                    const uint32_t i = b0 + (tid >> 1);
                    const bool rl = tid & 1u;
                    const bool on = i < e;
                    const uint32_t t = on ? E.TOPO[i] : 0u;
                    const uint32_t c0 = t & 0xFFFF, c1 = c0 + ((t >> 16) & 0xFF);
                    double* const A = rl ? E.R : E.D;
                    double x = on ? A[i] : 1.0;
                    for (uint32_t c = c0; c < c1; ++c) x = fma(-E.OFF[c], A[c], x);
                    const double ivd = rcpPivot(x);
                    const double iv = __shfl_sync(0xFFFFFFFFu, ivd, (tid & 31u) & ~1u);
                    const double y = (rl ? x : (on ? E.OFF[i] : 0.0)) * iv;
                    if (on) A[i] = y;
                } else {
                    for (uint32_t i = b0 + tid; i < e; i += nE) {
                        const uint32_t t = E.TOPO[i];
                        const uint32_t c0 = t & 0xFFFF, c1 = c0 + ((t >> 16) & 0xFF);
                        double d = E.D[i], r = E.R[i];
                        for (uint32_t c = c0; c < c1; ++c) {
                            const double oc = E.OFF[c];
                            d = fma(-oc, E.D[c], d);
                            r = fma(-oc, E.R[c], r);
                        }
                        const double iv = rcpPivot(d);
                        E.R[i] = r * iv;
                        E.D[i] = E.OFF[i] * iv;
                    }
                }
                groupSync(1, nE);
            }
        } else {
            for (uint32_t j = ga; j < F.nNodes; j += T) {
                const uint32_t i = F.nNodes - 1 - j;
                if (ga < b.nPf && j + T - ga < F.nNodes) {
                    const uint32_t hi = F.nNodes - (j + T - ga);
                    prefetchNodes(b, ga, F.node0 + (hi > T ? hi - T : 0), hi > T ? T : hi);
                }
                const uint32_t n = F.node0 + i;
                const uint32_t info = __ldg(b.nodeInfo + n);
                const unsigned long long stop = b.anyStop ? b.stopStep[__ldg(b.cellOf + n)] : ~0ull;
                const bool live = step < stop;
                const bool pending = s > 0 && step - 1 < stop;
                double d = 1.0, r = 0.0;
                if (info & kNodeCenter) {
                    if (live) d = __ldg(b.HS2 + n);
                } else if (live) {
                    assembleNode(b, n, info, pending, pending ? E.R[i] : 0.0, step, d, r);
                } else if (pending) {
                    updateNode(b, n, info, E.R[i]);
                }
                E.D[i] = d;
                E.R[i] = r;
                fenceCluster();
                atomicAdd(doneR0 + (E.TOPO[i] >> 24), 1u);
            }
        }
        clusterMeet(b, barR0, gen, kC, gaveUp);
        // the previous step's outputs (the update ran in this assembly), the
        // next step's SynChans, then rank 0 substitutes back
        if (rank == 0 && s > 0) forestOutputs(b, F, step - 1, tid, nth);
        if (s + 1 < nsteps)
            for (uint32_t k = k0 + gt; k < k1; k += GT) synapseStep(b, k, step + 1);
        if (rank == 0) {
            __syncthreads();
            for (uint32_t L = 0; L < F.nLevels; ++L) {
                const uint32_t e = lp[L + 1];
                for (uint32_t i = lp[L] + tid; i < e; i += nth) {
                    const uint32_t p = E.PAR[i];
                    double vm = E.R[i];
                    if (p != kNoParent) vm = fma(-E.D[i], E.R[p], vm);
                    E.R[i] = vm;
                }
                __syncthreads();
            }
            if (s + 1 < nsteps) {
                for (uint32_t L = tid; L < F.nLevels; L += nth) done[L] = 0;
                forestStimulus(b, F, step + 1);
            }
        }
        clusterMeet(b, barR0, gen, kC, gaveUp);
    }
    if (rank == 0) finishForest(b, F, f, E, step);
    clusterMeet(b, barR0, gen, kC, gaveUp);
}

// Forests of cluster blockIdx.x / kC (ctaPtr/ctaForests per cluster), each
// of at most `cap` nodes and kWsLevels - 1 levels (the host packs them so).
// Dynamic shared memory: kSmemLevels level offsets, kWsLevels counters, a
// barrier counter (4 words), then the forest's D and R (used in rank 0): a
// forest of at most `stageCap` nodes also gets OFF, TOPO and PAR there
// (30 B a node, like a one-CTA shared forest), a larger one keeps them in
// global memory (D and R only, 16 B a node, up to `cap` nodes).
__global__ void __launch_bounds__(1024, 1) hsForestStepMixedCluster(MixBatch b, const uint32_t* __restrict__ ctaPtr,
                                                                    const uint32_t* __restrict__ ctaForests,
                                                                    uint32_t kC, uint32_t cap, uint32_t stageCap,
                                                                    uint32_t elimWarps, uint32_t nsteps) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t* sLp = reinterpret_cast<uint32_t*>(smem);
    uint32_t* sDone = sLp + kSmemLevels;
    uint32_t* sBar = sDone + kWsLevels;
    double* sArea = reinterpret_cast<double*>(sBar + 4);
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    const uint32_t rank = cluster.block_rank();
    if (threadIdx.x == 0) *sBar = 0;
    for (uint32_t L = threadIdx.x; L < kWsLevels; L += blockDim.x) sDone[L] = 0;
    cluster.sync();                                   // rank 0's counters are set before anyone adds
    uint32_t* doneR0 = cluster.map_shared_rank(sDone, 0);
    uint32_t* barR0 = cluster.map_shared_rank(sBar, 0);
    uint32_t gen = 0;
    bool gaveUp = false;
    const uint32_t c = blockIdx.x / kC;
    for (uint32_t k = ctaPtr[c]; k < ctaPtr[c + 1]; ++k) {
        const MixForest F = b.forests[ctaForests[k]];
        const uint32_t* lp = b.levelPtr + F.level0;
        for (uint32_t i = threadIdx.x; i <= F.nLevels; i += blockDim.x) sLp[i] = lp[i];
        const bool stage = F.nNodes <= stageCap;
        double* sD = sArea;
        double* sR = sD + (stage ? stageCap : cap);
        double* sOff = sR + stageCap;
        uint32_t* sTopo = reinterpret_cast<uint32_t*>(sOff + stageCap);
        uint16_t* sPar = reinterpret_cast<uint16_t*>(sTopo + stageCap);
        Elim E;
        E.D = cluster.map_shared_rank(sD, 0);
        E.R = cluster.map_shared_rank(sR, 0);
        E.OFF = b.off + F.node0;
        E.TOPO = b.topo + F.node0;
        E.PAR = b.par + F.node0;
        if (stage && rank == 0) {
            for (uint32_t i = threadIdx.x; i < F.nNodes; i += blockDim.x) {
                sOff[i] = b.off[F.node0 + i];
                sTopo[i] = b.topo[F.node0 + i];
                sPar[i] = b.par[F.node0 + i];
            }
            E.OFF = sOff;
            E.TOPO = sTopo;
            E.PAR = sPar;
        }
        __syncthreads();
        stepForestCluster(b, F, ctaForests[k], E, sLp, sDone, doneR0, barR0, gen, rank, kC, elimWarps, nsteps,
                          gaveUp);
    }
    cluster.sync();                                   // rank 0's shared memory outlives every remote access
}

// One launch of the cluster kernel: nClusters clusters of kC CTAs.
cudaError_t launchForestStepMixedCluster(const MixBatch& b, const uint32_t* ctaPtr, const uint32_t* ctaForests,
                                         uint32_t nClusters, uint32_t kC, uint32_t threadsPerCta,
                                         uint32_t smemBytes, uint32_t cap, uint32_t stageCap, uint32_t elimWarps,
                                         uint32_t nsteps, cudaStream_t st) {
    cudaError_t e = cudaFuncSetAttribute(hsForestStepMixedCluster, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smemBytes);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nClusters * kC);
    cfg.blockDim = dim3(threadsPerCta);
    cfg.dynamicSmemBytes = smemBytes;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kC;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, hsForestStepMixedCluster, b, ctaPtr, ctaForests, kC, cap, stageCap, elimWarps,
                              nsteps);
}

cudaError_t launchForestStepMixed(const MixBatch& b, const uint32_t* ctaPtr, const uint32_t* ctaForests,
                                  uint32_t nCtas, uint32_t threadsPerCta, uint32_t smemBytes, uint32_t cap,
                                  uint32_t elimWarps, uint32_t nsteps, cudaStream_t st) {
    auto kern = b.anyStop ? hsForestStepMixed<true> : hsForestStepMixed<false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smemBytes);
    if (e != cudaSuccess) return e;
    kern<<<nCtas, threadsPerCta, smemBytes, st>>>(b, ctaPtr, ctaForests, cap, elimWarps, nsteps);
    return cudaGetLastError();
}

cudaError_t launchBatchReinitMixed(const MixBatch& b, uint32_t nNodes, const double* initVm, const float* k2x0,
                                   const uint32_t* evStart, cudaStream_t st) {
    hsReinitNodesMixed<<<(nNodes + 255) / 256, 256, 0, st>>>(b, nNodes, initVm, k2x0, evStart);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const uint32_t n = b.nCells > b.nForests ? b.nCells : b.nForests;
    hsReinitCellsMixed<<<(n + 127) / 128, 128, 0, st>>>(b);
    return cudaGetLastError();
}

}  // namespace hsg
