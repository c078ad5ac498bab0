// hs_mixed.cu -- mixed-precision batched HSolve step (sm_103a).
//
// One warp steps one cell; a warp owns a list of cells (packed by size on
// the host) and runs each for `nsteps` steps before moving on.  Per step:
//   tick 0   stimulus schedule (lane 0)
//   forward  levels deepest -> root.  A node at level L computes its own
//            channels (FP32 tables, gates, conductances; the K(Ca) 2-D gate;
//            its SynChans), assembles its FP64 matrix row, pulls the
//            eliminated rows of its children (FP64), and stores its
//            eliminated rhs and the reciprocal of its pivot.
//   backward levels root -> deepest: VMid = (rhs - off*VMid[parent])/pivot,
//            V = 2*VMid - V, then the node's Ca pools (HSolveActive::
//            advanceCalcium with VMid), FP32.
//   SpikeGens (lane 0), trace record.
// Reference routines: hsolve/HSolveActive.cpp:45-332, hsolve/HSolvePassive.cpp:
// 246-401 (same tree sweep, star form), biophysics/HHChannel2D.cpp:327-369,
// biophysics/SynChan.cpp:200-224, biophysics/SpikeGen.cpp:202-216.
#include <cuda_runtime.h>

#include "hs_mixed.cuh"

namespace hsg {

__constant__ ChanType c_chanTypes[kMaxChanTypes];
__constant__ C2dType c_c2dTypes[kMaxC2dTypes];
__constant__ SynType c_synTypes[kMaxSynTypes];

// Reciprocal of a positive FP64 pivot: FP32 hardware approximation as the
// seed, then two Newton-Raphson steps x <- x + x(1 - d x) in FP64 (each
// doubles the correct bits: ~2^-22 -> 2^-44 -> full precision).
__device__ __forceinline__ double rcpNewton(double d) {
    float f = __double2float_rn(d);
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(f));
    double x = (double)r;
    double e = fma(-d, x, 1.0);
    x = fma(x, e, x);
    e = fma(-d, x, 1.0);
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

__device__ __forceinline__ float gateF(const RowF& r, uint32_t nCol, int col, float x, float dt,
                                       float hdt, bool inst) {
    const float* ap = r.p + col;
    float2 a = *reinterpret_cast<const float2*>(ap);
    float2 b = *reinterpret_cast<const float2*>(ap + nCol);
    float C1 = fmaf(b.x - a.x, r.frac, a.x);
    float C2 = fmaf(b.y - a.y, r.frac, a.y);
    if (inst) return __fdividef(C1, C2);
    // The reference's trapezoidal step (x(2-T) + dt C1)/T with T = 1 + h,
    // h = dt/2 C2 (hsolve/HSolveActive.cpp:272-273), written as the
    // increment x + (dt C1 - 2 h x)/(1 + h): the same number in exact
    // arithmetic, but FP32 keeps the small h instead of rounding it into 1 + h.
    float h = hdt * C2;
    return x + __fdividef(fmaf(-2.0f * h, x, dt * C1), 1.0f + h);
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
    float2 z00 = *reinterpret_cast<const float2*>(p00);
    float2 z10 = make_float2(0.f, 0.f), z01 = z10, z11 = z10;
    if (!endX) z10 = *reinterpret_cast<const float2*>(p00 + 2 * ny);
    if (!endY) z01 = *reinterpret_cast<const float2*>(p00 + 2);
    if (!endX && !endY) z11 = *reinterpret_cast<const float2*>(p00 + 2 * ny + 2);
    float xFyF = xF * yF;
    float w00 = 1.f - xF - yF + xFyF, w10 = xF - xFyF, w01 = yF - xFyF;
    A = z00.x * w00 + z10.x * w10 + z01.x * w01 + z11.x * xFyF;
    B = z00.y * w00 + z10.y * w10 + z01.y * w01 + z11.y * xFyF;
}

// Channels, K(Ca), SynChans and matrix row of one compartment node.
__device__ __forceinline__ void nodeRow(const MixBatch& b, uint32_t n, unsigned long long step,
                                        double& diag, double& rhs) {
    const double V = b.V[n];
    const float v = (float)V;
    const float dt = b.dtf, hdt = 0.5f * b.dtf;
    RowF vr = rowF(b.vTab, b.vCol, b.vRows, v, b.vMin, b.vMax, b.vInvDx);
    float G = 0.f, GE = 0.f;
    const uint32_t p0 = b.pool0[n], p1 = b.pool0[n + 1];
    float cg[4] = {0.f, 0.f, 0.f, 0.f}, cge[4] = {0.f, 0.f, 0.f, 0.f};
    uint32_t s = b.state0[n];
    for (uint32_t q = b.chan0[n]; q < b.chan0[n + 1]; ++q) {
        const ChanType& t = c_chanTypes[b.chanType[q]];
        float frac = 1.f;
        if (t.xp) {
            float x = gateF(vr, b.vCol, t.colX, b.state[s], dt, hdt, t.instant & 1);
            b.state[s++] = x;
            frac *= powi(x, t.xp, t.xpf);
        }
        if (t.yp) {
            float y = gateF(vr, b.vCol, t.colY, b.state[s], dt, hdt, t.instant & 2);
            b.state[s++] = y;
            frac *= powi(y, t.yp, t.ypf);
        }
        if (t.zp) {
            float z;
            if (t.zSrc >= 0) {
                RowF cr = rowF(b.caTab, b.caCol, b.caRows, b.poolCa[p0 + t.zSrc], b.caMin, b.caMax, b.caInvDx);
                z = gateF(cr, b.caCol, t.colZ, b.state[s], dt, hdt, t.instant & 4);
            } else {
                z = gateF(vr, b.vCol, t.colZ, b.state[s], dt, hdt, t.instant & 4);
            }
            b.state[s++] = z;
            frac *= powi(z, t.zp, t.zpf);
        }
        float gk = b.chanGbar[q] * frac;
        b.chanGk[q] = gk;
        G += gk;
        GE = fmaf(gk, t.ek, GE);
        if (t.caTarget >= 0 && t.caTarget < 4) {
            cg[t.caTarget] += gk;
            cge[t.caTarget] = fmaf(gk, t.ek, cge[t.caTarget]);
        }
    }
    for (uint32_t p = p0; p < p1 && p - p0 < 4; ++p) {
        b.caG[p] = cg[p - p0];
        b.caGE[p] = cge[p - p0];
    }
    // K(Ca) and other HHChannel2D: inputs are Vm and Ca of the previous step
    for (uint32_t k = b.c2d0[n]; k < b.c2d0[n + 1]; ++k) {
        const C2dType& t = c_c2dTypes[b.c2dType[k]];
        float c1 = t.conc1 >= 0 ? b.poolCa[p0 + t.conc1] : 0.f;
        float c2 = t.conc2 >= 0 ? b.poolCa[p0 + t.conc2] : 0.f;
        float x = t.dep0 == 0 ? v : t.dep0 == 1 ? c1 : t.dep0 == 2 ? c2 : 0.f;
        float y = t.dep1 == 0 ? v : t.dep1 == 1 ? c1 : t.dep1 == 2 ? c2 : 0.f;
        float A, B;
        interp2dF(b.g2d + b.g2dOff[t.gate], b.g2dGeom + 6 * t.gate, b.g2dN[2 * t.gate],
                  b.g2dN[2 * t.gate + 1], x, y, A, B);
        float X = b.c2dX[k];
        if (t.instant & 1) X = __fdividef(A, B);
        else if (B > 1.0e-10f) {
            // HHChannelBase::integrate, X e + (A/B)(1 - e) with e = exp(-B dt),
            // as X + (A/B - X)(1 - e) with 1 - e = -expm1(-B dt) (no cancellation)
            float em = -expm1f(-B * dt);
            X = fmaf(__fdividef(A, B) - X, em, X);
        } else X = fmaf(A, dt, X);
        b.c2dX[k] = X;
        float gk = b.c2dGbar[k] * powi(X, t.xp, t.xpf);
        G += gk;
        GE = fmaf(gk, t.ek, GE);
    }
    // SynChans: events delivered this step (SimpleSynHandler), dual exponential
    for (uint32_t k = b.syn0[n]; k < b.syn0[n + 1]; ++k) {
        const SynType& t = c_synTypes[b.synType[k]];
        uint32_t e = b.evCur[k];
        const uint32_t end = b.evEnd[k];
        float act = 0.f;
        while (e < end && b.evStep[e] <= step) act += b.evAct[e++];
        b.evCur[k] = e;
        float X = fmaf(act, t.xc1, b.synX[k] * t.xc2);
        float Y = fmaf(X, t.yc1, b.synY[k] * t.yc2);
        b.synX[k] = X;
        b.synY[k] = Y;
        float gk = Y * b.synNorm[k];
        G += gk;
        GE = fmaf(gk, t.ek, GE);
    }
    diag = b.HS2[n] + (double)G;
    rhs = fma(V, b.CmByDt[n], b.EmByRm[n]) + (double)GE;
}

__device__ void stepCellMixed(const MixBatch& b, uint32_t cell, uint32_t nsteps, uint32_t lane) {
    const MixCellRange cr = b.cells[cell];
    const uint32_t* lp = b.levelPtr + cr.level0;
    const uint32_t base = cr.node0;
    unsigned long long step = b.stepCount[cell];
    uint32_t stimCur = b.stimCur[cell];
    uint32_t spk = b.spikeCount[cell];
    for (uint32_t s = 0; s < nsteps; ++s, ++step) {
        if (lane == 0) {
            while (stimCur < cr.nStim && b.stimStep[cr.stim0 + stimCur] <= step) {
                b.injVal[cr.inj0 + b.stimEntry[cr.stim0 + stimCur]] = b.stimValue[cr.stim0 + stimCur];
                ++stimCur;
            }
        }
        __syncwarp();
        // assembly: every compartment's channels and FP64 row, in parallel;
        // the row is staged in inv (pivot) and rhsF (right-hand side)
        for (uint32_t i = lane; i < cr.nNodes; i += 32) {
            const uint32_t n = base + i;
            const uint32_t info = b.nodeInfo[n];
            if (info & kNodeCenter) continue;
            double d, r;
            nodeRow(b, n, step, d, r);
            if (info & kNodeInject)
                for (uint32_t k = 0; k < cr.nInj; ++k)
                    if (b.injNode[cr.inj0 + k] == i) r += b.injVal[cr.inj0 + k];
            b.inv[n] = d;
            b.rhsF[n] = r;
        }
        __syncwarp();
        // forward elimination, deepest level first: pull the children's
        // eliminated rows, keep 1/pivot and the eliminated rhs
        for (int L = (int)cr.nLevels - 1; L >= 0; --L) {
            for (uint32_t i = lp[L] + lane; i < lp[L + 1]; i += 32) {
                const uint32_t n = base + i;
                const bool center = b.nodeInfo[n] & kNodeCenter;
                double d = center ? b.HS2[n] : b.inv[n];
                double r = center ? 0.0 : b.rhsF[n];
                for (uint32_t c = b.child0[n]; c < b.child0[n + 1]; ++c) {
                    const double oc = b.off[c];
                    const double f = oc * b.inv[c];
                    d = fma(-f, oc, d);
                    r = fma(-f, b.rhsF[c], r);
                }
                b.inv[n] = rcpNewton(d);
                b.rhsF[n] = r;
            }
            __syncwarp();
        }
        // backward substitution, root first; then V and the Ca pools
        for (uint32_t L = 0; L < cr.nLevels; ++L) {
            for (uint32_t i = lp[L] + lane; i < lp[L + 1]; i += 32) {
                const uint32_t n = base + i;
                double r = b.rhsF[n];
                if (L > 0) r = fma(-b.off[n], b.VMid[b.parent[n]], r);
                const double vm = r * b.inv[n];
                b.VMid[n] = vm;
                if (!(b.nodeInfo[n] & kNodeCenter)) {
                    const double Vold = b.V[n];
                    const double Vnew = fma(2.0, vm, -Vold);
                    b.V[n] = Vnew;
                    const float vca = (float)(b.caAdvance == 1 ? vm : fma(2.0, vm, -Vnew));
                    for (uint32_t p = b.pool0[n]; p < b.pool0[n + 1]; ++p) {
                        float act = fmaf(-b.caG[p], vca, b.caGE[p]);
                        // c f1 + f2 act with f1 = 1 - g1 (g1 = 1 - f1 from FP64)
                        float c0 = b.poolC[p];
                        float c = fmaf(-b.poolF1[p], c0, c0) + b.poolF2[p] * act;
                        float ca = b.poolBasal[p] + c;
                        if (b.poolCeil[p] > 0.f && ca > b.poolCeil[p]) { ca = b.poolCeil[p]; c = ca - b.poolBasal[p]; }
                        if (ca < b.poolFloor[p]) { ca = b.poolFloor[p]; c = ca - b.poolBasal[p]; }
                        b.poolC[p] = c;
                        b.poolCa[p] = ca;
                    }
                }
            }
            __syncwarp();
        }
        // SpikeGens (SpikeGen::process with the HSolve's V and currTime)
        if (lane == 0) {
            const double currTime = b.dt * (double)(step + 1);
            for (uint32_t k = cr.sg0; k < cr.sg0 + cr.nSg; ++k) {
                double Vs = b.V[base + b.sgNode[k]];
                if (Vs > (double)b.sgThresh[k]) {
                    if ((float)(currTime + b.dt / 2.0) >= b.sgLast[k] + b.sgRefract[k]) {
                        if (!(b.sgEdge[k] && b.sgFired[k])) {
                            if (spk < b.spikeCap) {
                                b.spikeGen[(size_t)cell * b.spikeCap + spk] = k - cr.sg0;
                                b.spikeTime[(size_t)cell * b.spikeCap + spk] = (float)currTime;
                            }
                            ++spk;
                            b.sgLast[k] = (float)currTime;
                            b.sgFired[k] = 1;
                        }
                    }
                } else {
                    b.sgFired[k] = 0;
                }
            }
        }
        if (cr.nRec && ((step + 1) % b.recStride) == 0) {
            uint32_t smp = (uint32_t)((step + 1) / b.recStride);
            if (smp < b.recCap)
                for (uint32_t r = lane; r < cr.nRec; r += 32)
                    b.recBuf[(size_t)smp * b.recLd + cr.rec0 + r] = b.V[base + b.recNode[cr.rec0 + r]];
        }
        __syncwarp();
    }
    if (lane == 0) {
        b.stepCount[cell] = step;
        b.stimCur[cell] = stimCur;
        b.spikeCount[cell] = spk;
    }
}

__global__ void __launch_bounds__(512) hsBatchStepMixed(MixBatch b, const uint32_t* __restrict__ warpCellPtr,
                                                        const uint32_t* __restrict__ warpCells,
                                                        uint32_t nWarps, uint32_t nsteps) {
    uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t lane = threadIdx.x & 31;
    if (w >= nWarps) return;
    for (uint32_t k = warpCellPtr[w]; k < warpCellPtr[w + 1]; ++k) stepCellMixed(b, warpCells[k], nsteps, lane);
}

// Reinit: V = initVm, gates at their steady state, Ca = CaBasal, synapses,
// K(Ca) X, spike and stimulus state.  One warp per cell.
__global__ void hsBatchReinitMixed(MixBatch b, const double* __restrict__ initVm,
                                   const float* __restrict__ c2dX0, const uint32_t* __restrict__ evStart) {
    uint32_t cell = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t lane = threadIdx.x & 31;
    if (cell >= b.nCells) return;
    const MixCellRange cr = b.cells[cell];
    for (uint32_t i = lane; i < cr.nNodes; i += 32) {
        uint32_t n = cr.node0 + i;
        b.V[n] = initVm[n];
        for (uint32_t p = b.pool0[n]; p < b.pool0[n + 1]; ++p) {
            b.poolC[p] = 0.f;
            b.poolCa[p] = b.poolBasal[p];
        }
    }
    __syncwarp();
    for (uint32_t i = lane; i < cr.nNodes; i += 32) {
        uint32_t n = cr.node0 + i;
        if (b.nodeInfo[n] & kNodeCenter) continue;
        float v = (float)b.V[n];
        RowF vr = rowF(b.vTab, b.vCol, b.vRows, v, b.vMin, b.vMax, b.vInvDx);
        uint32_t s = b.state0[n];
        uint32_t p0 = b.pool0[n];
        for (uint32_t q = b.chan0[n]; q < b.chan0[n + 1]; ++q) {
            const ChanType& t = c_chanTypes[b.chanType[q]];
            if (t.xp) b.state[s++] = gateF(vr, b.vCol, t.colX, 0.f, 0.f, 0.f, true);
            if (t.yp) b.state[s++] = gateF(vr, b.vCol, t.colY, 0.f, 0.f, 0.f, true);
            if (t.zp) {
                if (t.zSrc >= 0) {
                    RowF cr2 = rowF(b.caTab, b.caCol, b.caRows, b.poolCa[p0 + t.zSrc], b.caMin, b.caMax, b.caInvDx);
                    b.state[s++] = gateF(cr2, b.caCol, t.colZ, 0.f, 0.f, 0.f, true);
                } else {
                    b.state[s++] = gateF(vr, b.vCol, t.colZ, 0.f, 0.f, 0.f, true);
                }
            }
        }
        for (uint32_t k = b.c2d0[n]; k < b.c2d0[n + 1]; ++k) b.c2dX[k] = c2dX0[k];
        for (uint32_t k = b.syn0[n]; k < b.syn0[n + 1]; ++k) {
            b.synX[k] = 0.f;
            b.synY[k] = 0.f;
            b.evCur[k] = evStart[k];
        }
    }
    for (uint32_t k = cr.sg0 + lane; k < cr.sg0 + cr.nSg; k += 32) b.sgLast[k] = -b.sgRefract[k];
    if (lane == 0) {
        b.stepCount[cell] = 0;
        b.stimCur[cell] = 0;
        b.spikeCount[cell] = 0;
    }
    if (cr.nRec)
        for (uint32_t r = lane; r < cr.nRec; r += 32)
            b.recBuf[cr.rec0 + r] = b.V[cr.node0 + b.recNode[cr.rec0 + r]];
}

// Scatter of host-supplied inject values to their solver slots.
__global__ void hsScatterInject(double* const* __restrict__ addr, uint8_t* const* __restrict__ flag,
                                const double* __restrict__ val, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    *addr[i] = val[i];
    if (flag[i]) *flag[i] = 1;
}

cudaError_t launchScatterInject(double* const* addr, uint8_t* const* flag, const double* val, uint32_t n,
                                cudaStream_t st) {
    if (!n) return cudaSuccess;
    hsScatterInject<<<(n + 255) / 256, 256, 0, st>>>(addr, flag, val, n);
    return cudaGetLastError();
}

cudaError_t uploadMixedTypes(const ChanType* ct, int nct, const C2dType* kt, int nkt, const SynType* st,
                             int nst, cudaStream_t s) {
    cudaError_t e = cudaSuccess;
    if (nct) e = cudaMemcpyToSymbolAsync(c_chanTypes, ct, nct * sizeof(ChanType), 0, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && nkt)
        e = cudaMemcpyToSymbolAsync(c_c2dTypes, kt, nkt * sizeof(C2dType), 0, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && nst)
        e = cudaMemcpyToSymbolAsync(c_synTypes, st, nst * sizeof(SynType), 0, cudaMemcpyHostToDevice, s);
    return e;
}

cudaError_t launchBatchStepMixed(const MixBatch& b, const uint32_t* warpCellPtr, const uint32_t* warpCells,
                                 uint32_t nWarps, uint32_t nsteps, uint32_t threadsPerCta, cudaStream_t st) {
    uint32_t blocks = (nWarps * 32 + threadsPerCta - 1) / threadsPerCta;
    hsBatchStepMixed<<<blocks, threadsPerCta, 0, st>>>(b, warpCellPtr, warpCells, nWarps, nsteps);
    return cudaGetLastError();
}

cudaError_t launchBatchReinitMixed(const MixBatch& b, const double* initVm, const float* c2dX0,
                                   const uint32_t* evStart, cudaStream_t st) {
    uint32_t blocks = (b.nCells * 32 + 255) / 256;
    hsBatchReinitMixed<<<blocks ? blocks : 1, 256, 0, st>>>(b, initVm, c2dX0, evStart);
    return cudaGetLastError();
}

}  // namespace hsg
