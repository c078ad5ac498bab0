// hs_mixed.cu -- mixed-precision batched HSolve step (sm_103a).
//
// A team of W warps steps one cell at a time; every team owns a list of
// cells (packed by cost on the host) and runs each for `nsteps` steps before
// moving on.  A team synchronises with a named barrier (bar.sync id, 32*W),
// or __syncwarp when W = 1.  Per step:
//   tick 0    stimulus schedule
//   assembly  every compartment node, in parallel over the team: FP32 rate
//             lookup and gate update for each channel slot, conductances,
//             the K(Ca) 2-D gate, SynChans; FP64 matrix row.
//   forward   work units level by level (hs_mixed.cuh), each unit serially
//             by one thread: pull the children's eliminated rows
//             (diag -= off^2/pivot_c, rhs -= off*g_c), keep 1/pivot and
//             g = rhs/pivot (FP64).
//   backward  the same units in reverse: VMid = g - (off/pivot)*VMid[parent],
//             V = 2*VMid - V, then the node's Ca pool (FP32).
//   SpikeGens, trace record.
// Reference routines: hsolve/HSolveActive.cpp:45-332, hsolve/HSolvePassive.cpp:
// 246-401 (the same elimination, tree form), biophysics/HHChannel2D.cpp:327-369,
// biophysics/SynChan.cpp:200-224, synapse/SimpleSynHandler.cpp:98-113,
// biophysics/SpikeGen.cpp:202-216.
#include <cuda_runtime.h>

#include "hs_mixed.cuh"

namespace hsg {

__constant__ ChanType c_chanTypes[kMaxChanTypes];
__constant__ C2dType c_c2dTypes[kMaxC2dTypes];
__constant__ SynType c_synTypes[kMaxSynTypes];

// Reciprocal of a positive FP64 pivot: the FP32 hardware approximation
// (relative error below 2^-22) refined by one Newton-Raphson step
// x <- x + x(1 - d x) in FP64, which squares the error (below 2^-44).
__device__ __forceinline__ double rcpNewton(double d) {
    float f = __double2float_rn(d);
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(f));
    double x = (double)r;
    double e = fma(-d, x, 1.0);
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

// Channels, K(Ca), SynChans and FP64 matrix row of one compartment node.
__device__ __forceinline__ void nodeRow(const MixBatch& b, uint32_t n, uint32_t info,
                                        unsigned long long step, double& diag, double& rhs) {
    const uint64_t ld = b.ld;
    const double V = b.V[n];
    const uint32_t types = b.ctype4[n];
    const float v = (float)V;
    const float dt = b.dtf, hdt = 0.5f * b.dtf;
    const float ca = (info & kNodePool) ? b.poolCa[n] : 0.f;
    RowF vr = rowF(b.vTab, b.vCol, b.vRows, v, b.vMin, b.vMax, b.vInvDx);
    float G = 0.f, GE = 0.f, cg = 0.f, cge = 0.f;
#pragma unroll
    for (int j = 0; j < kMaxChan; ++j) {
        const uint32_t tj = (types >> (8 * j)) & 0xFF;
        if (tj == kNoType) break;
        const ChanType& t = c_chanTypes[tj];
        float frac = 1.f;
        float* st = b.state + (uint64_t)(3 * j) * ld + n;
        if (t.xp) {
            float x = gateF(vr, b.vCol, t.colX, st[0], dt, hdt, t.instant & 1);
            st[0] = x;
            frac *= powi(x, t.xp, t.xpf);
        }
        if (t.yp) {
            float y = gateF(vr, b.vCol, t.colY, st[ld], dt, hdt, t.instant & 2);
            st[ld] = y;
            frac *= powi(y, t.yp, t.ypf);
        }
        if (t.zp) {
            float z;
            if (t.zCa) {
                RowF cr = rowF(b.caTab, b.caCol, b.caRows, ca, b.caMin, b.caMax, b.caInvDx);
                z = gateF(cr, b.caCol, t.colZ, st[2 * ld], dt, hdt, t.instant & 4);
            } else {
                z = gateF(vr, b.vCol, t.colZ, st[2 * ld], dt, hdt, t.instant & 4);
            }
            st[2 * ld] = z;
            frac *= powi(z, t.zp, t.zpf);
        }
        const float gk = b.gbar[(uint64_t)j * ld + n] * frac;
        G += gk;
        GE = fmaf(gk, t.ek, GE);
        if (t.caTarget) {
            cg += gk;
            cge = fmaf(gk, t.ek, cge);
        }
    }
    if (info & kNodePool) {
        b.caG[n] = cg;
        b.caGE[n] = cge;
    }
    // HHChannel2D (K(Ca)): inputs are Vm and Ca of the previous step
    const uint32_t k2 = (info >> 8) & 0xFF;
    if (k2 != kNoType) {
        const C2dType& t = c_c2dTypes[k2];
        float x = t.dep0 == 0 ? v : t.dep0 == 1 ? ca : 0.f;
        float y = t.dep1 == 0 ? v : t.dep1 == 1 ? ca : 0.f;
        float A, B;
        interp2dF(b.g2d + b.g2dOff[t.gate], b.g2dGeom + 6 * t.gate, b.g2dN[2 * t.gate],
                  b.g2dN[2 * t.gate + 1], x, y, A, B);
        float X = b.k2x[n];
        if (t.instant & 1) X = __fdividef(A, B);
        else if (B > 1.0e-10f) {
            // HHChannelBase::integrate, X e + (A/B)(1 - e) with e = exp(-B dt),
            // as X + (A/B - X)(1 - e), 1 - e = -expm1(-B dt) (no cancellation)
            float em = -expm1f(-B * dt);
            X = fmaf(__fdividef(A, B) - X, em, X);
        } else X = fmaf(A, dt, X);
        b.k2x[n] = X;
        float gk = b.k2gbar[n] * powi(X, t.xp, t.xpf);
        G += gk;
        GE = fmaf(gk, t.ek, GE);
    }
    // SynChans: events delivered this step (SimpleSynHandler), dual exponential
    if (info & kNodeSyn) {
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
    }
    diag = b.HS2[n] + (double)G;
    rhs = fma(V, b.CmByDt[n], b.EmByRm[n]) + (double)GE;
}

struct Team {
    uint32_t tid, nth, bar;
};

__device__ __forceinline__ void teamSync(const Team& t) {
    if (t.nth == 32) __syncwarp();
    else asm volatile("bar.sync %0, %1;" ::"r"(t.bar), "r"(t.nth) : "memory");
}

__device__ void stepCell(const MixBatch& b, uint32_t cell, uint32_t nsteps, const Team& tm) {
    const MixCellRange cr = b.cells[cell];
    const uint32_t base = cr.node0;
    unsigned long long step = b.stepCount[cell];
    uint32_t stimCur = b.stimCur[cell];
    uint32_t spk = b.spikeCount[cell];
    for (uint32_t s = 0; s < nsteps; ++s, ++step) {
        if (tm.tid == 0) {
            while (stimCur < cr.nStim && b.stimStep[cr.stim0 + stimCur] <= step) {
                b.injVal[cr.inj0 + b.stimEntry[cr.stim0 + stimCur]] = b.stimValue[cr.stim0 + stimCur];
                ++stimCur;
            }
        }
        teamSync(tm);
        // assembly, all compartment nodes in parallel; rows staged in inv/gEl
        for (uint32_t i = tm.tid; i < cr.nNodes; i += tm.nth) {
            const uint32_t n = base + i;
            const uint32_t info = b.nodeInfo[n];
            if (info & kNodeCenter) {
                b.inv[n] = b.HS2[n];
                b.gEl[n] = 0.0;
                continue;
            }
            double d, r;
            nodeRow(b, n, info, step, d, r);
            if (info & kNodeInject)
                for (uint32_t k = 0; k < cr.nInj; ++k)
                    if (b.injNode[cr.inj0 + k] == i) r += b.injVal[cr.inj0 + k];
            b.inv[n] = d;
            b.gEl[n] = r;
        }
        teamSync(tm);
        // forward elimination: units level by level, each unit serially;
        // every node pulls its children (diag -= off^2/pivot_c, rhs -= off*g_c)
        const uint32_t* up = b.unitPtr + cr.level0;
        const uint2* un = b.units + cr.unit0;
        const uint32_t* cl = b.childList + cr.child0;
        for (uint32_t L = 0; L < cr.nLevels; ++L) {
            for (uint32_t u = up[L] + tm.tid; u < up[L + 1]; u += tm.nth) {
                const uint2 rg = un[u];
                // the node eliminated just before is the last child in
                // post-order and the lower neighbour in a chain: its pivot
                // and g stay in registers
                double pIv = 0.0, pG = 0.0;
                for (uint32_t v = rg.x; v < rg.y; ++v) {
                    const uint32_t n = base + v;
                    double d = b.inv[n], r = b.gEl[n];
                    const uint32_t cs = b.childStart[n], nc = (b.nodeInfo[n] >> 16) & 0xFF;
                    for (uint32_t k = cs; k < cs + nc; ++k) {
                        const uint32_t cv = cl[k];
                        const uint32_t c = base + cv;
                        const bool prev = cv + 1 == v && v > rg.x;
                        const double ivc = prev ? pIv : b.inv[c];
                        const double gc = prev ? pG : b.gEl[c];
                        d = fma(-b.offsq[c], ivc, d);
                        r = fma(-b.off[c], gc, r);
                    }
                    pIv = rcpNewton(d);
                    pG = r * pIv;
                    b.inv[n] = pIv;
                    b.gEl[n] = pG;
                }
            }
            teamSync(tm);
        }
        // back substitution in the reverse order: VMid = g - (off/pivot) VMid[parent],
        // V = 2 VMid - V, then the node's Ca pool
        for (int L = (int)cr.nLevels - 1; L >= 0; --L) {
            for (uint32_t u = up[L] + tm.tid; u < up[L + 1]; u += tm.nth) {
                const uint2 rg = un[u];
                double pVm = 0.0;   // VMid of the node substituted just before
                for (uint32_t v = rg.y; v-- > rg.x;) {
                    const uint32_t n = base + v;
                    double vm = b.gEl[n];
                    const uint32_t pa = b.parent[n];
                    if (pa != ~0u) {
                        const double vp = (pa == v + 1 && v + 1 < rg.y) ? pVm : b.VMid[base + pa];
                        vm = fma(-(b.off[n] * b.inv[n]), vp, vm);
                    }
                    pVm = vm;
                    b.VMid[n] = vm;
                    const uint32_t info = b.nodeInfo[n];
                    if (!(info & kNodeCenter)) {
                        const double Vold = b.V[n];
                        const double Vnew = fma(2.0, vm, -Vold);
                        b.V[n] = Vnew;
                        if (info & kNodePool) {
                            const float vca = (float)(b.caAdvance == 1 ? vm : fma(2.0, vm, -Vnew));
                            float act = fmaf(-b.caG[n], vca, b.caGE[n]);
                            // c f1 + f2 act with f1 = 1 - g1 (g1 = 1 - f1 from FP64)
                            float c0v = b.poolC[n];
                            float c = fmaf(-b.poolG1[n], c0v, c0v) + b.poolF2[n] * act;
                            float cav = b.poolBasal[n] + c;
                            if (b.poolCeil[n] > 0.f && cav > b.poolCeil[n]) { cav = b.poolCeil[n]; c = cav - b.poolBasal[n]; }
                            if (cav < b.poolFloor[n]) { cav = b.poolFloor[n]; c = cav - b.poolBasal[n]; }
                            b.poolC[n] = c;
                            b.poolCa[n] = cav;
                        }
                    }
                }
            }
            teamSync(tm);
        }
        // SpikeGens (SpikeGen::process with the solver's V and currTime)
        if (tm.tid == 0) {
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
                for (uint32_t r = tm.tid; r < cr.nRec; r += tm.nth)
                    b.recBuf[(size_t)smp * b.recLd + cr.rec0 + r] = b.V[base + b.recNode[cr.rec0 + r]];
        }
        teamSync(tm);
    }
    if (tm.tid == 0) {
        b.stepCount[cell] = step;
        b.stimCur[cell] = stimCur;
        b.spikeCount[cell] = spk;
    }
}

__global__ void __launch_bounds__(512) hsBatchStepMixed(MixBatch b, const uint32_t* __restrict__ teamCellPtr,
                                                        const uint32_t* __restrict__ teamCells, uint32_t nTeams,
                                                        uint32_t warpsPerTeam, uint32_t nsteps) {
    const uint32_t teamsPerCta = blockDim.x / (32 * warpsPerTeam);
    const uint32_t teamInCta = threadIdx.x / (32 * warpsPerTeam);
    const uint32_t team = blockIdx.x * teamsPerCta + teamInCta;
    if (team >= nTeams) return;     // whole teams leave together
    Team tm;
    tm.nth = 32 * warpsPerTeam;
    tm.tid = threadIdx.x - teamInCta * tm.nth;
    tm.bar = teamInCta + 1;
    for (uint32_t k = teamCellPtr[team]; k < teamCellPtr[team + 1]; ++k) stepCell(b, teamCells[k], nsteps, tm);
}

// Reinit: V = initVm, gates at their steady state, Ca = CaBasal, synapses,
// K(Ca) X, spike and stimulus state.  One warp per cell.
__global__ void hsBatchReinitMixed(MixBatch b, const double* __restrict__ initVm,
                                   const float* __restrict__ k2x0, const uint32_t* __restrict__ evStart) {
    uint32_t cell = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t lane = threadIdx.x & 31;
    if (cell >= b.nCells) return;
    const MixCellRange cr = b.cells[cell];
    const uint64_t ld = b.ld;
    for (uint32_t i = lane; i < cr.nNodes; i += 32) {
        const uint32_t n = cr.node0 + i;
        const uint32_t info = b.nodeInfo[n];
        b.V[n] = initVm[n];
        if (info & kNodeCenter) continue;
        if (info & kNodePool) {
            b.poolC[n] = 0.f;
            b.poolCa[n] = b.poolBasal[n];
        }
        const float ca = (info & kNodePool) ? b.poolCa[n] : 0.f;
        RowF vr = rowF(b.vTab, b.vCol, b.vRows, (float)b.V[n], b.vMin, b.vMax, b.vInvDx);
        const uint32_t types = b.ctype4[n];
        for (int j = 0; j < kMaxChan; ++j) {
            const uint32_t tj = (types >> (8 * j)) & 0xFF;
            if (tj == kNoType) break;
            const ChanType& t = c_chanTypes[tj];
            float* st = b.state + (uint64_t)(3 * j) * ld + n;
            if (t.xp) st[0] = gateF(vr, b.vCol, t.colX, 0.f, 0.f, 0.f, true);
            if (t.yp) st[ld] = gateF(vr, b.vCol, t.colY, 0.f, 0.f, 0.f, true);
            if (t.zp) {
                if (t.zCa) {
                    RowF cr2 = rowF(b.caTab, b.caCol, b.caRows, ca, b.caMin, b.caMax, b.caInvDx);
                    st[2 * ld] = gateF(cr2, b.caCol, t.colZ, 0.f, 0.f, 0.f, true);
                } else {
                    st[2 * ld] = gateF(vr, b.vCol, t.colZ, 0.f, 0.f, 0.f, true);
                }
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
    for (uint32_t k = cr.sg0 + lane; k < cr.sg0 + cr.nSg; k += 32) {
        b.sgLast[k] = -b.sgRefract[k];
        b.sgFired[k] = 0;
    }
    if (lane == 0) {
        b.stepCount[cell] = 0;
        b.stimCur[cell] = 0;
        b.spikeCount[cell] = 0;
    }
    __syncwarp();
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

cudaError_t launchBatchStepMixed(const MixBatch& b, const uint32_t* teamCellPtr, const uint32_t* teamCells,
                                 uint32_t nTeams, uint32_t warpsPerTeam, uint32_t threadsPerCta, uint32_t nsteps,
                                 cudaStream_t st) {
    uint32_t teamsPerCta = threadsPerCta / (32 * warpsPerTeam);
    uint32_t blocks = (nTeams + teamsPerCta - 1) / teamsPerCta;
    hsBatchStepMixed<<<blocks, threadsPerCta, 0, st>>>(b, teamCellPtr, teamCells, nTeams, warpsPerTeam, nsteps);
    return cudaGetLastError();
}

cudaError_t launchBatchReinitMixed(const MixBatch& b, const double* initVm, const float* k2x0,
                                   const uint32_t* evStart, cudaStream_t st) {
    uint32_t blocks = (b.nCells * 32 + 255) / 256;
    hsBatchReinitMixed<<<blocks ? blocks : 1, 256, 0, st>>>(b, initVm, k2x0, evStart);
    return cudaGetLastError();
}

}  // namespace hsg
