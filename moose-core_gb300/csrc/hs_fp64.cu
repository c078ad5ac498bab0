// hs_fp64.cu -- the FP64 drop-in HSolve step on GB300 (sm_103a).
//
// One CTA steps one cell for `nsteps` clock steps without returning to the
// host.  Per step, in the reference's tick order (scheduling/Clock.cpp:872-921):
//   tick 0   basal-inject schedule
//   tick 1/4 SimpleSynHandler -> SynChan, HHChannel2D  (one thread per object)
//   tick 6   HSolveActive::step (hsolve/HSolveActive.cpp:45-66):
//            advanceChannels + calculateChannelCurrents + updateMatrix
//            (one thread per compartment), forward elimination and back
//            substitution (level by level over the pull programs, the rows
//            of a level shared by the CTA; cable runs by one thread),
//            advanceCalcium (one thread per pool), SpikeGens, trace record.
// Compiled with --fmad=false: every operation is the reference's IEEE
// operation in the reference's order, so Vm/Ca are bit-identical to the CPU
// HSolve wherever no libm call is involved (exp/log only in HHChannel2D and
// non-integer gate powers).
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "../../include/moose_gb300.h"
#include "hs_device.cuh"
#include "hs_plan.h"

namespace hsg {

// ---- tick 1: external calcium (DifShell, DifBuffer, MMPump) ----------------
// biophysics/DifShell.cpp, biophysics/DifBuffer.cpp, biophysics/MMPump.cpp.
// The objects process in tick order and each send reaches its targets at
// once (a target later in the same tick sees this step's value), so one
// thread walks them in order.  State: kDifState arrays of nDif (see DevCell).
namespace dif {
constexpr double kF = 96485.3415;                 // DifShell::F
constexpr double kEpsilon = 1.0e-10;              // DifShell/DifBuffer::EPSILON
constexpr double kPi = 3.14159265358979323846;    // M_PI
enum { C_ = 0, PREVC, DC, CM, BFREE, BBOUND, PREVFREE, AF, BF, ACT, VOL, OUTERA, INNERA };
}  // namespace dif

__device__ __forceinline__ double& difS(const DevCell& c, int field, uint32_t k) {
    return c.difState[(size_t)field * c.nDif + k];
}
__device__ __forceinline__ double difP(const DevCell& c, uint32_t k, int i) {
    return c.difPar[(size_t)k * HS_DIF_NPAR + i];
}

// DifShell::calculateVolumeArea, DifBuffer::vReinit's geometry
__device__ void difGeometry(const DevCell& c, uint32_t k) {
    using namespace dif;
    const int shape = (int)difP(c, k, 4);
    const double length = difP(c, k, 5), diameter = difP(c, k, 6), thickness = difP(c, k, 7);
    const double rOut = diameter / 2.;
    double rIn = rOut - thickness;
    if (rIn < 0) rIn = 0.;
    if (shape == 0) {
        if (length == 0.0) {
            difS(c, VOL, k) = 4. / 3. * kPi * (rOut * rOut * rOut - rIn * rIn * rIn);
            difS(c, OUTERA, k) = 4 * kPi * rOut * rOut;
            difS(c, INNERA, k) = 4 * kPi * rIn * rIn;
        } else {
            difS(c, VOL, k) = (kPi * length) * (rOut * rOut - rIn * rIn);
            difS(c, OUTERA, k) = 2 * kPi * rOut * length;
            difS(c, INNERA, k) = 2 * kPi * rIn * length;
        }
    } else if (shape == 1) {
        difS(c, VOL, k) = kPi * diameter * diameter * thickness / 4.0;
        difS(c, OUTERA, k) = kPi * diameter * diameter / 4.0;
        difS(c, INNERA, k) = difS(c, OUTERA, k);
    } else {
        difS(c, VOL, k) = difP(c, k, 8);
        difS(c, OUTERA, k) = difP(c, k, 9);
        difS(c, INNERA, k) = difP(c, k, 10);
    }
}

__device__ __forceinline__ double difIntegrate(double state, double dt, double A, double B) {
    if (B > dif::kEpsilon) {
        const double x = exp(-B * dt);
        return state * x + (A / B) * (1 - x);
    }
    return state + A * dt;
}

// inner/outerDifSourceOut of object s: fluxFromIn/Out of each target
__device__ void difSendFlux(const DevCell& c, uint32_t s, int kind, double value, double thickness) {
    using namespace dif;
    const uint32_t slot = s * kDifMsgKinds + kind;
    for (uint32_t i = c.difOff[slot]; i < c.difOff[slot + 1]; ++i) {
        const uint32_t t = c.difDst[i];
        const bool shell = c.difKind[t] == HS_DIF_SHELL;
        const double D = shell ? difP(c, t, 1) : difP(c, t, 3);
        const double area = kind == HS_DMSG_OUTER ? difS(c, OUTERA, t) : difS(c, INNERA, t);
        const double tt = difP(c, t, 7);
        if (shell) {
            const double diff = 2. * D / difS(c, VOL, t) * area / (thickness + tt);
            difS(c, DC, t) += diff * value;
            difS(c, CM, t) += diff;
        } else {
            const double d = 2 * D / difS(c, VOL, t) * area / (tt + thickness);
            difS(c, AF, t) += d * value;
            difS(c, BF, t) += d;
        }
    }
}

// concentrationOut of shell s: HHChannel concen (HSolve::addConc) and DifBuffer
// concentration (its activation)
__device__ void difSendConc(const DevCell& c, uint32_t s, double C) {
    uint32_t slot = s * kDifMsgKinds + HS_DMSG_CONC_CHAN;
    for (uint32_t i = c.difOff[slot]; i < c.difOff[slot + 1]; ++i) c.extCa[c.difDst[i]] = C;
    slot = s * kDifMsgKinds + HS_DMSG_CONC_BUF;
    for (uint32_t i = c.difOff[slot]; i < c.difOff[slot + 1]; ++i) difS(c, dif::ACT, c.difDst[i]) = C;
}

// DifShell::vReinit, DifBuffer::vReinit (MMPump::reinit does nothing)
__device__ void difReinit(const DevCell& c) {
    using namespace dif;
    for (uint32_t k = 0; k < c.nDif; ++k) {
        const int kind = c.difKind[k];
        if (kind == HS_DIF_SHELL) {
            difS(c, DC, k) = difP(c, k, 3);
            difS(c, CM, k) = 0;
            difGeometry(c, k);
            difS(c, C_, k) = difP(c, k, 0);
            difS(c, PREVC, k) = difP(c, k, 0);
            difSendConc(c, k, difS(c, C_, k));
            difSendFlux(c, k, HS_DMSG_INNER, difS(c, PREVC, k), difP(c, k, 7));
            difSendFlux(c, k, HS_DMSG_OUTER, difS(c, PREVC, k), difP(c, k, 7));
        } else if (kind == HS_DIF_BUFFER) {
            difS(c, AF, k) = 0;
            difS(c, BF, k) = 0;
            difGeometry(c, k);
            const double bTot = difP(c, k, 0), kf = difP(c, k, 1), kb = difP(c, k, 2);
            difS(c, BFREE, k) = bTot / (1 + difS(c, ACT, k) * kf / kb);
            difS(c, PREVFREE, k) = difS(c, BFREE, k);
            difS(c, BBOUND, k) = bTot - difS(c, BFREE, k);
            difSendFlux(c, k, HS_DMSG_INNER, difS(c, PREVFREE, k), difP(c, k, 7));
            difSendFlux(c, k, HS_DMSG_OUTER, difS(c, PREVFREE, k), difP(c, k, 7));
        }
    }
}

// DifShell::vProcess, DifBuffer::vProcess, MMPump::process
__device__ void difProcess(const DevCell& c) {
    using namespace dif;
    for (uint32_t k = 0; k < c.nDif; ++k) {
        const int kind = c.difKind[k];
        if (kind == HS_DIF_SHELL) {
            difS(c, C_, k) = difIntegrate(difS(c, C_, k), c.dt, difS(c, DC, k), difS(c, CM, k));
            difS(c, DC, k) = difP(c, k, 3);
            difS(c, CM, k) = 0;
            difS(c, PREVC, k) = difS(c, C_, k);
            difSendFlux(c, k, HS_DMSG_INNER, difS(c, PREVC, k), difP(c, k, 7));
            difSendFlux(c, k, HS_DMSG_OUTER, difS(c, PREVC, k), difP(c, k, 7));
            difSendConc(c, k, difS(c, C_, k));
        } else if (kind == HS_DIF_BUFFER) {
            const double bTot = difP(c, k, 0), kf = difP(c, k, 1), kb = difP(c, k, 2);
            difS(c, AF, k) += kb * difS(c, BBOUND, k);
            difS(c, BF, k) += kf * difS(c, ACT, k);
            difS(c, BFREE, k) = difIntegrate(difS(c, BFREE, k), c.dt, difS(c, AF, k), difS(c, BF, k));
            difS(c, BBOUND, k) = bTot - difS(c, BFREE, k);
            difS(c, PREVFREE, k) = difS(c, BFREE, k);
            difSendFlux(c, k, HS_DMSG_INNER, difS(c, PREVFREE, k), difP(c, k, 7));
            difSendFlux(c, k, HS_DMSG_OUTER, difS(c, PREVFREE, k), difP(c, k, 7));
            const uint32_t slot = k * kDifMsgKinds + HS_DMSG_REACTION;     // reactionOut -> DifShell::vBuffer
            for (uint32_t i = c.difOff[slot]; i < c.difOff[slot + 1]; ++i) {
                const uint32_t t = c.difDst[i];
                difS(c, DC, t) += kb * difS(c, BBOUND, k);
                difS(c, CM, t) += kf * difS(c, BFREE, k);
            }
            difS(c, AF, k) = 0;
            difS(c, BF, k) = 0;
        } else {
            const double vMax = difP(c, k, 0), Kd = difP(c, k, 1);
            const uint32_t slot = k * kDifMsgKinds + HS_DMSG_PUMP;          // PumpOut -> DifShell::vMMPump
            for (uint32_t i = c.difOff[slot]; i < c.difOff[slot + 1]; ++i) {
                const uint32_t t = c.difDst[i];
                difS(c, CM, t) += (vMax / difS(c, VOL, t)) / (difS(c, C_, t) + Kd);
            }
        }
    }
}

// HSolveActive::sendValues, IkOut (hsolve/HSolveActive.cpp:367-376):
// (Ek - Vm) Gk of each channel, channel order, to DifShell::vInflux
__device__ void difSendIk(const DevCell& c) {
    for (uint32_t q = 0; q < c.C; ++q) {
        if (c.ikOff[q] == c.ikOff[q + 1]) continue;
        const double I = (c.Ek[q] - c.V[c.chanCompt[q]]) * c.Gk[q];
        for (uint32_t i = c.ikOff[q]; i < c.ikOff[q + 1]; ++i) {
            const uint32_t t = c.ikDst[i];
            difS(c, dif::DC, t) += I / (dif::kF * difP(c, t, 2) * difS(c, dif::VOL, t));
        }
    }
}

// ---- tick 1/4: external objects -------------------------------------------
__device__ __forceinline__ void synchanStep(const DevCell& c, uint32_t k, double currTime) {
    // SimpleSynHandler::vProcess: deliver events with time <= currTime
    double activation = 0.0;
    uint32_t e = c.evCur[k], end = c.evPtr[k + 1];
    while (e < end && c.evTime[e] <= currTime) {
        activation += c.evW[e] / c.dt;
        ++e;
    }
    c.evCur[k] = e;
    double act = c.synAct[k];
    if (activation != 0.0) act += activation;
    // SynChan::calcGk
    double X = act * c.synXc1[k] + c.synX[k] * c.synXc2[k];
    double Y = X * c.synYc1[k] + c.synY[k] * c.synYc2[k];
    c.synX[k] = X;
    c.synY[k] = Y;
    c.synAct[k] = 0.0;
    c.synGk[k] = Y * c.synNorm[k] * c.synMod[k];
}

__device__ __forceinline__ double depValue(int dep, double vm, double c1, double c2) {
    return dep == 0 ? vm : dep == 1 ? c1 : dep == 2 ? c2 : 0.0;
}

__device__ __forceinline__ void chan2dStep(const DevCell& c, uint32_t k) {
    double g = c.c2dGbar[k];
    double xp = c.c2dXpow[k];
    if (xp > 0) {
        int gi = c.c2dGate[k];
        double vm = c.c2dVm[k], c1 = c.c2dC1[k], c2 = c.c2dC2[k];
        double x = depValue(c.c2dDep0[k], vm, c1, c2);
        double y = depValue(c.c2dDep1[k], vm, c1, c2);
        double A, B;
        interp2dBoth(c.g2dAB + c.g2dOff[gi], c.g2dGeom + 6 * gi, c.g2dN[2 * gi],
                     c.g2dN[2 * gi + 1], x, y, A, B);
        double X = c.c2dX[k];
        if (c.c2dInstant[k] & 1) {
            X = A / B;
        } else if (B > 1.0e-10) {   // HHChannelBase::integrate (exponential Euler)
            double e = exp(-B * c.dt);
            X = X * e + (A / B) * (1 - e);
        } else {
            X = X + A * c.dt;
        }
        c.c2dX[k] = X;
        g *= takePower(X, xp);
    }
    c.c2dGk[k] = g * c.c2dMod[k];
}

// ---- tick 6, per compartment: channels + matrix row -----------------------
__device__ __forceinline__ void comptStep(const DevCell& c, uint32_t ic) {
    double V = c.V[ic];
    Row vRow = tableRow(V, c.vMin, c.vMax, c.vDx, c.vCol);
    double GkSum = 0.0, GkEkSum = 0.0;
    for (uint32_t q = c.chanPtr[ic]; q < c.chanPtr[ic + 1]; ++q) {
        int32_t s = c.stateOff[q];
        int inst = c.instant[q];
        double fraction = c.mod[q];
        double C1, C2;
        double xp = c.Xpow[q], yp = c.Ypow[q], zp = c.Zpow[q];
        double xs = 0, ys = 0, zs = 0;
        if (xp > 0.0) {
            tableLookup(c.vTab, c.vCol, c.colX[q], vRow, C1, C2);
            xs = gateStep(c.state[s], C1, C2, c.dt, inst & 1);
            c.state[s++] = xs;
        }
        if (yp > 0.0) {
            tableLookup(c.vTab, c.vCol, c.colY[q], vRow, C1, C2);
            ys = gateStep(c.state[s], C1, C2, c.dt, inst & 2);
            c.state[s++] = ys;
        }
        if (zp > 0.0) {
            int32_t src = c.zSrc[q];
            if (src >= 0) {
                Row r = tableRow(c.ca[src], c.caMin, c.caMax, c.caDx, c.caCol);
                tableLookup(c.caTab, c.caCol, c.colZ[q], r, C1, C2);
            } else if (c.extCa[q] > 0) {
                Row r = tableRow(c.extCa[q], c.caMin, c.caMax, c.caDx, c.caCol);
                tableLookup(c.caTab, c.caCol, c.colZ[q], r, C1, C2);
            } else {
                tableLookup(c.vTab, c.vCol, c.colZ[q], vRow, C1, C2);
            }
            zs = gateStep(c.state[s], C1, C2, c.dt, inst & 4);
            c.state[s] = zs;
        }
        // ChannelStruct::process
        if (xp > 0.0) fraction *= takePower(xs, xp);
        if (yp > 0.0) fraction *= takePower(ys, yp);
        if (zp > 0.0) fraction *= takePower(zs, zp);
        double gk = c.Gbar[q] * fraction;
        c.Gk[q] = gk;
        GkSum += gk;
        GkEkSum += gk * c.Ek[q];
    }
    // external conductances in tick-4 send order (HSolve::addGkEk)
    double eg = c.ext[2 * ic], ege = c.ext[2 * ic + 1];
    for (uint32_t k = c.extPtr[ic]; k < c.extPtr[ic + 1]; ++k) {
        int32_t code = c.extList[k];
        double gk = code >= 0 ? c.c2dGk[code] : c.synGk[-code - 1];
        double ek = code >= 0 ? c.c2dEk[code] : c.synEk[-code - 1];
        eg += gk;
        ege += gk * ek;
    }
    c.prevExt[2 * ic] = eg;
    c.prevExt[2 * ic + 1] = ege;
    // HSolveActive::updateMatrix
    const uint32_t N = c.N;
    double diag = c.HS2[ic] + GkSum;
    double rhs = V * c.CmByDt[ic] + c.EmByRm[ic] + GkEkSum;
    if (c.injPresent[ic]) rhs += c.injVarying[ic] + c.injBasal[ic];
    diag += eg;
    rhs += ege;
    c.M[ic] = diag;
    c.M[N + ic] = rhs;
}

// ---- elimination -------------------------------------------------------------
// A level costs the eliminating warp ~150 instructions of index loads and
// loop control around its few FP64 operations, all on one dependency chain.
// A run of cable rows (one row per level, see CellPlan::fRun/bRun) is walked
// by lane 0 alone with the pivot's values carried in registers, the row
// indices computed (row r: diagonal M[r], right-hand side M[N + r],
// off-diagonal to r + 1 at M[2N + H + r]) and the next row's operands loaded
// ahead; the operations and their order are those of the general loop.
__device__ __forceinline__ void forwardCableRun(const DevCell& c, uint32_t r, uint32_t run) {
    double* M = c.M;
    const uint32_t N = c.N, offBase = 2 * N + c.H;
    double d = M[r - 1], rhs = M[N + r - 1];
    double off = M[offBase + r - 1], dNext = M[r], rNext = M[N + r];
    for (uint32_t i = 0; i < run; ++i, ++r) {
        const double o = off, dr = dNext, rr = rNext;
        if (i + 1 < run) {
            off = M[offBase + r];
            dNext = M[r + 1];
            rNext = M[N + r + 1];
        }
        const double q = o / d;
        d = dr - q * o;
        rhs = rr - q * rhs;
        M[r] = d;
        M[N + r] = rhs;
    }
}

__device__ __forceinline__ void backwardCableRun(const DevCell& c, uint32_t i, uint32_t run) {
    const double* M = c.M;
    const uint32_t N = c.N, offBase = 2 * N + c.H;
    double vNext = c.VMid[i + 1];
    double rhs = M[N + i], off = M[offBase + i], diag = M[i], vOld = c.V[i];
    for (uint32_t j = 0; j < run; ++j, --i) {
        const double r = rhs, o = off, dg = diag, vo = vOld;
        if (j + 1 < run) {
            rhs = M[N + i - 1];
            off = M[offBase + i - 1];
            diag = M[i - 1];
            vOld = c.V[i - 1];
        }
        double v = r;
        v -= o * vNext;
        v /= dg;
        c.VMid[i] = v;
        c.V[i] = 2 * v - vo;
        vNext = v;
    }
}

template <bool WARP>
__device__ __forceinline__ void levelSync() {
    if (WARP) __syncwarp();
    else __syncthreads();
}

// Forward elimination and back substitution by a group of `nth` threads:
// one warp per cell in the FP64 batch, the whole CTA in the drop-in (the
// rows of a level are independent, so a wide level of a branched cell is
// shared by all warps instead of walked by one; a barrier per level).
template <bool WARP>
__device__ __forceinline__ void eliminate(const DevCell& c, uint32_t tid, uint32_t nth) {
    double* M = c.M;
    // Waves (CellPlan::fWavePtr): the level programs' updates, each wave's
    // on disjoint entries, so the group shares a wave update by update
    // instead of walking a row's chain per thread.  With a whole CTA, a
    // thread's first update of the next wave (read-only descriptors) is
    // loaded before the barrier.
    if (WARP) {
        for (uint32_t w = 0; w < c.fWaves; ++w) {
            for (uint32_t k = c.fWavePtr[w] + tid; k < c.fWavePtr[w + 1]; k += nth) {
                const int4 x = c.fWaveOps[2 * k], y = c.fWaveOps[2 * k + 1];
                const double q = M[y.x] / M[y.y];
                M[x.x] -= q * M[x.y];
                if (x.z >= 0) M[x.z] -= q * M[x.w];
            }
            levelSync<WARP>();
        }
    } else if (c.fWaves) {
        uint32_t kb = c.fWavePtr[0] + tid, ke = c.fWavePtr[1];
        int4 xn = make_int4(0, 0, -1, 0), yn = make_int4(0, 0, 0, 0);
        if (kb < ke) {
            xn = c.fWaveOps[2 * kb];
            yn = c.fWaveOps[2 * kb + 1];
        }
        for (uint32_t w = 0; w < c.fWaves; ++w) {
            const uint32_t k0 = kb, e = ke;
            const int4 x0 = xn, y0 = yn;
            if (w + 1 < c.fWaves) {
                kb = c.fWavePtr[w + 1] + tid;
                ke = c.fWavePtr[w + 2];
                if (kb < ke) {
                    xn = c.fWaveOps[2 * kb];
                    yn = c.fWaveOps[2 * kb + 1];
                }
            }
            if (k0 < e) {
                const double q = M[y0.x] / M[y0.y];
                M[x0.x] -= q * M[x0.y];
                if (x0.z >= 0) M[x0.z] -= q * M[x0.w];
            }
            for (uint32_t k = k0 + nth; k < e; k += nth) {
                const int4 x = c.fWaveOps[2 * k], y = c.fWaveOps[2 * k + 1];
                const double q = M[y.x] / M[y.y];
                M[x.x] -= q * M[x.y];
                if (x.z >= 0) M[x.z] -= q * M[x.w];
            }
            levelSync<WARP>();
        }
    }
    for (uint32_t l = 0; l < (c.fWaves ? 0u : c.fLevels); ++l) {
        if (const uint32_t run = c.fRun[l]) {
            if (tid == 0) forwardCableRun(c, c.fRunRow[l], run);
            levelSync<WARP>();
            l += run - 1;
            continue;
        }
        for (uint32_t k = c.fLevelPtr[l] + tid; k < c.fLevelPtr[l + 1]; k += nth) {
            // t -= l / pivot * a.  A row's consecutive updates by one pivot
            // (its diagonal and right-hand side: the reference computes
            // HS[4i+1] / HS[4i] for both) share the quotient: it is computed
            // once, the same IEEE division of the same operands, which takes
            // one FP64 division off each level of the dependency chain.
            int32_t ql = -1, qp = -1;
            double q = 0.0;
            for (uint32_t o = c.fOpPtr[k]; o < c.fOpPtr[k + 1]; ++o) {
                int4 op = c.fOps[o];
                if (op.y != ql || op.w != qp) {
                    q = M[op.y] / M[op.w];
                    ql = op.y;
                    qp = op.w;
                }
                M[op.x] -= q * M[op.z];
                if (op.x == ql || op.x == qp) ql = -1;   // an operand changed
            }
        }
        levelSync<WARP>();
    }
    // Back substitution.  With a whole CTA, a thread's first row of the next
    // level has its index, right-hand side, diagonal, old V and term range
    // (none of which this level writes) loaded before the barrier; the level
    // then waits only on the VMid values its terms read.
    const uint32_t N = c.N;
    if (WARP) {
        for (uint32_t l = 0; l < c.bLevels; ++l) {
            if (const uint32_t run = c.bRun[l]) {
                if (tid == 0) backwardCableRun(c, c.bRunRow[l], run);
                levelSync<WARP>();
                l += run - 1;
                continue;
            }
            for (uint32_t k = c.bLevelPtr[l] + tid; k < c.bLevelPtr[l + 1]; k += nth) {
                uint32_t i = c.bRows[k];
                double v = M[N + i];
                for (uint32_t t = c.bTermPtr[k]; t < c.bTermPtr[k + 1]; ++t) {
                    int2 term = c.bTerms[t];
                    v -= M[term.x] * c.VMid[term.y];
                }
                v /= M[i];
                c.VMid[i] = v;
                c.V[i] = 2 * v - c.V[i];
            }
            levelSync<WARP>();
        }
        return;
    }
    uint32_t nk = 0, ne = 0, ni = 0, nt0 = 0, nt1 = 0;
    double nr = 0.0, nd = 1.0, nv = 0.0;
    auto preload = [&](uint32_t l) {
        nk = c.bLevelPtr[l] + tid;
        ne = c.bLevelPtr[l + 1];
        if (nk < ne) {
            ni = c.bRows[nk];
            nr = M[N + ni];
            nd = M[ni];
            nv = c.V[ni];
            nt0 = c.bTermPtr[nk];
            nt1 = c.bTermPtr[nk + 1];
        }
    };
    bool ahead = false;
    for (uint32_t l = 0; l < c.bLevels; ++l) {
        if (const uint32_t run = c.bRun[l]) {
            if (tid == 0) backwardCableRun(c, c.bRunRow[l], run);
            levelSync<WARP>();
            l += run - 1;
            ahead = false;
            continue;
        }
        if (!ahead) preload(l);
        const uint32_t k0 = nk, e = ne, i0 = ni, t0 = nt0, t1 = nt1;
        const double r0 = nr, d0 = nd, v0 = nv;
        ahead = l + 1 < c.bLevels && !c.bRun[l + 1];
        if (ahead) preload(l + 1);
        if (k0 < e) {
            double v = r0;
            for (uint32_t t = t0; t < t1; ++t) {
                int2 term = c.bTerms[t];
                v -= M[term.x] * c.VMid[term.y];
            }
            v /= d0;
            c.VMid[i0] = v;
            c.V[i0] = 2 * v - v0;
        }
        for (uint32_t k = k0 + nth; k < e; k += nth) {
            uint32_t i = c.bRows[k];
            double v = M[N + i];
            for (uint32_t t = c.bTermPtr[k]; t < c.bTermPtr[k + 1]; ++t) {
                int2 term = c.bTerms[t];
                v -= M[term.x] * c.VMid[term.y];
            }
            v /= M[i];
            c.VMid[i] = v;
            c.V[i] = 2 * v - c.V[i];
        }
        levelSync<WARP>();
    }
}

// ---- advanceCalcium, per pool ----------------------------------------------
__device__ __forceinline__ void poolStep(const DevCell& c, uint32_t p) {
    double act = c.iCa[p];
    for (uint32_t f = c.feedPtr[p]; f < c.feedPtr[p + 1]; ++f) {
        uint32_t q = c.feedChan[f];
        uint32_t ic = c.chanCompt[q];
        double v = c.caAdvance == 1 ? c.VMid[ic] : (2 * c.VMid[ic] - c.V[ic]);
        act += c.Gk[q] * (c.Ek[q] - v);
    }
    double cc = c.f1[p] * c.c[p] + c.f2[p] * act;
    double ca = c.CaBasal[p] + cc;
    if (c.ceil[p] > 0 && ca > c.ceil[p]) {
        ca = c.ceil[p];
        cc = ca - c.CaBasal[p];
    }
    if (ca < c.floor_[p]) {
        ca = c.floor_[p];
        cc = ca - c.CaBasal[p];
    }
    c.c[p] = cc;
    c.ca[p] = ca;
    c.iCa[p] = 0.0;
}

// One cell, `nsteps` steps, executed by a group of `nth` threads (a whole
// CTA for the drop-in, one warp for the batch).  `barrier` orders the phases.
template <bool WARP>
__device__ __forceinline__ void groupSync() {
    if (WARP) __syncwarp();
    else __syncthreads();
}

template <bool WARP>
__device__ void stepCell(const DevCell& c, uint32_t nsteps, uint32_t tid, uint32_t nth) {
    unsigned long long step = c.ctl->nSteps;
    uint32_t stimPtr = c.ctl->stimPtr, nSpikes = c.ctl->nSpikes, nSamples = c.ctl->nSamples;
    groupSync<WARP>();
    for (uint32_t s = 0; s < nsteps; ++s, ++step) {
        const double currTime = c.dt * (double)(step + 1);   // Clock: dt_ * endStep
        if (tid == 0) {
            while (stimPtr < c.nStim && c.stimStep[stimPtr] <= step) {
                uint32_t h = c.stimCompt[stimPtr];
                c.injPresent[h] = 1;
                c.injBasal[h] = c.stimValue[stimPtr];
                ++stimPtr;
            }
            if (c.nDif) difProcess(c);     // tick 1, before the gates read extCa
        }
        for (uint32_t k = tid; k < c.S; k += nth) synchanStep(c, k, currTime);
        for (uint32_t k = tid; k < c.K2; k += nth) chan2dStep(c, k);
        groupSync<WARP>();
        for (uint32_t h = tid; h < c.H; h += nth) c.M[2 * c.N + h] = c.HJ0[h];
        for (uint32_t ic = tid; ic < c.N; ic += nth) comptStep(c, ic);
        groupSync<WARP>();
        eliminate<WARP>(c, tid, nth);
        groupSync<WARP>();
        for (uint32_t p = tid; p < c.P; p += nth) poolStep(c, p);
        groupSync<WARP>();
        if (tid == 0 && c.nDif) difSendIk(c);
        // sendValues for the next step's tick-4 objects; SpikeGens; traces
        for (uint32_t k = tid; k < c.K2; k += nth) {
            c.c2dVm[k] = c.V[c.c2dCompt[k]];
            if (c.c2dConc1[k] >= 0) c.c2dC1[k] = c.ca[c.c2dConc1[k]];
            if (c.c2dConc2[k] >= 0) c.c2dC2[k] = c.ca[c.c2dConc2[k]];
        }
        if (tid == 0) {
            for (uint32_t k = 0; k < c.SG; ++k) {
                double V = c.V[c.sgCompt[k]];
                if (V > c.sgThreshold[k]) {
                    if ((currTime + c.dt / 2.0) >= (c.sgLast[k] + c.sgRefract[k])) {
                        if (!(c.sgEdge[k] && c.sgFired[k])) {
                            if (nSpikes < c.spikeCap) {
                                c.spikeGen[nSpikes] = k;
                                c.spikeTime[nSpikes] = currTime;
                            }
                            ++nSpikes;
                            c.sgLast[k] = currTime;
                            c.sgFired[k] = 1;
                        }
                    }
                } else {
                    c.sgFired[k] = 0;
                }
            }
        }
        if (c.nRec && ((step + 1) % c.recStride) == 0) {
            if (nSamples < c.recCap)
                for (uint32_t r = tid; r < c.nRec; r += nth)
                    c.recBuf[(size_t)nSamples * c.recLd + r] = recValue(c, c.recCompt[r]);
            ++nSamples;
        }
        for (uint32_t ic = tid; ic < c.N; ic += nth) {
            c.injVarying[ic] = 0.0;
            c.ext[2 * ic] = 0.0;
            c.ext[2 * ic + 1] = 0.0;
        }
        groupSync<WARP>();
    }
    if (tid == 0) {
        c.ctl->nSteps = step;
        c.ctl->stimPtr = stimPtr;
        c.ctl->nSpikes = nSpikes;
        c.ctl->nSamples = nSamples;
    }
}

__global__ void __launch_bounds__(256, 1) hsStepFp64(DevCell c, uint32_t nsteps) {
    stepCell<false>(c, nsteps, threadIdx.x, blockDim.x);
}

// One cell stepped by a thread-block cluster.  On one SM a large cell's step
// is bound by the FP64 work of its channels and matrix rows (one SM's FP64
// pipe); the cluster's CTAs share that work -- object k goes to thread k of
// the cluster -- and the wide waves and levels of the elimination
// (eliminateCluster), while rank 0's CTA walks the narrow ones.
// Every object's arithmetic is unchanged and the phases keep their order,
// so the results are bit-identical to stepCell.  The hardware cluster
// barrier (release/acquire at cluster scope) orders the phases; all data
// stays in the cell's global arena.
// One fused forward update and one back-substitution row, as eliminate does
// them.
__device__ __forceinline__ void waveUpdate(const DevCell& c, double* M, uint32_t k) {
    const int4 x = c.fWaveOps[2 * k], y = c.fWaveOps[2 * k + 1];
    const double q = M[y.x] / M[y.y];
    M[x.x] -= q * M[x.y];
    if (x.z >= 0) M[x.z] -= q * M[x.w];
}

__device__ __forceinline__ void backRow(const DevCell& c, const double* M, uint32_t N, uint32_t k) {
    uint32_t i = c.bRows[k];
    double v = M[N + i];
    for (uint32_t t = c.bTermPtr[k]; t < c.bTermPtr[k + 1]; ++t) {
        int2 term = c.bTerms[t];
        v -= M[term.x] * c.VMid[term.y];
    }
    v /= M[i];
    c.VMid[i] = v;
    c.V[i] = 2 * v - c.V[i];
}

// The elimination of a cell stepped by a cluster.  A forward wave or a
// back-substitution level of at least kClusterWide updates or rows is
// shared by all the cluster's CTAs, a cluster barrier after it (and before
// it, when rank 0 wrote alone since the last one); narrower ones are
// walked by rank 0's CTA with a CTA barrier, as eliminate walks them.  The
// updates of a wave, and the rows of a level, are independent, so which
// thread of which CTA does one changes nothing: bit-identical to
// eliminate.  Every CTA takes the same branches (they depend on the sizes
// alone), so all meet at every cluster barrier.  Cells without waves (the
// cable runs' level programs) and cells below kClusterElimRows compartments
// are eliminated by rank 0 alone, as eliminate does it: sharing pays from
// ~4,000 compartments on (one GB300, 8 CTAs: 5,000 compartments 407 -> 378
// us per step, 10,000: 631 -> 498), and costs below (1,000: 171 -> 190,
// 2,000: 231 -> 244; the shared waves' cluster barriers and the L2 reads
// after them outweigh the work they split).
constexpr uint32_t kClusterWide = 1024;
constexpr uint32_t kClusterElimRows = 4096;

__device__ void eliminateCluster(const DevCell& c, cooperative_groups::cluster_group& cl, uint32_t rank,
                                 uint32_t tid, uint32_t nth, uint32_t g, uint32_t G) {
    if (!c.fWaves || c.N < kClusterElimRows) {
        if (rank == 0) eliminate<false>(c, tid, nth);
        return;
    }
    double* M = c.M;
    bool alone = false;      // rank 0 wrote since the last cluster barrier
    for (uint32_t w = 0; w < c.fWaves; ++w) {
        const uint32_t b0 = c.fWavePtr[w], e = c.fWavePtr[w + 1];
        if (e - b0 >= kClusterWide) {
            if (alone) cl.sync();
            alone = false;
            for (uint32_t k = b0 + g; k < e; k += G) waveUpdate(c, M, k);
            cl.sync();
        } else {
            if (rank == 0) {
                for (uint32_t k = b0 + tid; k < e; k += nth) waveUpdate(c, M, k);
                __syncthreads();
            }
            alone = true;
        }
    }
    const uint32_t N = c.N;
    for (uint32_t l = 0; l < c.bLevels; ++l) {
        if (const uint32_t run = c.bRun[l]) {
            if (rank == 0) {
                if (tid == 0) backwardCableRun(c, c.bRunRow[l], run);
                __syncthreads();
            }
            alone = true;
            l += run - 1;
            continue;
        }
        const uint32_t b0 = c.bLevelPtr[l], e = c.bLevelPtr[l + 1];
        if (e - b0 >= kClusterWide) {
            if (alone) cl.sync();
            alone = false;
            for (uint32_t k = b0 + g; k < e; k += G) backRow(c, M, N, k);
            cl.sync();
        } else {
            if (rank == 0) {
                for (uint32_t k = b0 + tid; k < e; k += nth) backRow(c, M, N, k);
                __syncthreads();
            }
            alone = true;
        }
    }
}

__device__ void stepCellCluster(const DevCell& c, uint32_t nsteps) {
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    const uint32_t rank = cl.block_rank();
    const uint32_t tid = threadIdx.x, nth = blockDim.x;
    const uint32_t g = rank * nth + tid, G = cl.num_blocks() * nth;
    unsigned long long step = c.ctl->nSteps;
    uint32_t stimPtr = c.ctl->stimPtr, nSpikes = c.ctl->nSpikes, nSamples = c.ctl->nSamples;
    cl.sync();
    for (uint32_t s = 0; s < nsteps; ++s, ++step) {
        const double currTime = c.dt * (double)(step + 1);
        if (g == 0) {
            while (stimPtr < c.nStim && c.stimStep[stimPtr] <= step) {
                uint32_t h = c.stimCompt[stimPtr];
                c.injPresent[h] = 1;
                c.injBasal[h] = c.stimValue[stimPtr];
                ++stimPtr;
            }
            if (c.nDif) difProcess(c);
        }
        for (uint32_t k = g; k < c.S; k += G) synchanStep(c, k, currTime);
        for (uint32_t k = g; k < c.K2; k += G) chan2dStep(c, k);
        cl.sync();
        for (uint32_t h = g; h < c.H; h += G) c.M[2 * c.N + h] = c.HJ0[h];
        for (uint32_t ic = g; ic < c.N; ic += G) comptStep(c, ic);
        cl.sync();
        eliminateCluster(c, cl, rank, tid, nth, g, G);
        cl.sync();
        for (uint32_t p = g; p < c.P; p += G) poolStep(c, p);
        cl.sync();
        if (g == 0 && c.nDif) difSendIk(c);
        for (uint32_t k = g; k < c.K2; k += G) {
            c.c2dVm[k] = c.V[c.c2dCompt[k]];
            if (c.c2dConc1[k] >= 0) c.c2dC1[k] = c.ca[c.c2dConc1[k]];
            if (c.c2dConc2[k] >= 0) c.c2dC2[k] = c.ca[c.c2dConc2[k]];
        }
        if (g == 0) {
            for (uint32_t k = 0; k < c.SG; ++k) {
                double V = c.V[c.sgCompt[k]];
                if (V > c.sgThreshold[k]) {
                    if ((currTime + c.dt / 2.0) >= (c.sgLast[k] + c.sgRefract[k])) {
                        if (!(c.sgEdge[k] && c.sgFired[k])) {
                            if (nSpikes < c.spikeCap) {
                                c.spikeGen[nSpikes] = k;
                                c.spikeTime[nSpikes] = currTime;
                            }
                            ++nSpikes;
                            c.sgLast[k] = currTime;
                            c.sgFired[k] = 1;
                        }
                    }
                } else {
                    c.sgFired[k] = 0;
                }
            }
        }
        if (c.nRec && ((step + 1) % c.recStride) == 0) {
            if (nSamples < c.recCap)
                for (uint32_t r = g; r < c.nRec; r += G)
                    c.recBuf[(size_t)nSamples * c.recLd + r] = recValue(c, c.recCompt[r]);
            ++nSamples;
        }
        for (uint32_t ic = g; ic < c.N; ic += G) {
            c.injVarying[ic] = 0.0;
            c.ext[2 * ic] = 0.0;
            c.ext[2 * ic + 1] = 0.0;
        }
        cl.sync();
    }
    if (g == 0) {
        c.ctl->nSteps = step;
        c.ctl->stimPtr = stimPtr;
        c.ctl->nSpikes = nSpikes;
        c.ctl->nSamples = nSamples;
    }
}

__global__ void __launch_bounds__(256, 1) hsStepFp64Cluster(DevCell c, uint32_t nsteps) {
    stepCellCluster(c, nsteps);
}

// Separate drop-in solvers stepped in one launch (hs_process_group): CTA k
// steps solver k exactly as hsStepFp64 steps it alone; in the cluster form
// cluster k steps solver k exactly as hsStepFp64Cluster does.
__global__ void __launch_bounds__(256) hsGroupStepFp64(const DevCell* __restrict__ cells, uint32_t nsteps) {
    stepCell<false>(cells[blockIdx.x], nsteps, threadIdx.x, blockDim.x);
}

__global__ void __launch_bounds__(256) hsGroupStepFp64Cluster(const DevCell* __restrict__ cells, uint32_t nsteps) {
    stepCellCluster(cells[blockIdx.x / cooperative_groups::this_cluster().num_blocks()], nsteps);
}

// Batched FP64.  A CTA either steps its cells one after the other with all
// its threads, as the drop-in steps one cell (ctaCellPtr gives it a
// non-empty list: the largest cells, whose chains would otherwise bound the
// step), or runs one warp per cell on the cells listed per warp.  Both
// forms do the drop-in's arithmetic in its order: results are bit-identical
// whichever form steps a cell.
__global__ void __launch_bounds__(256) hsBatchStepFp64(const DevCell* __restrict__ cells,
                                                       const uint32_t* __restrict__ warpCellPtr,
                                                       const uint32_t* __restrict__ warpCells,
                                                       uint32_t nWarps, const uint32_t* __restrict__ ctaCellPtr,
                                                       const uint32_t* __restrict__ ctaCells, uint32_t nsteps) {
    const uint32_t c0 = ctaCellPtr[blockIdx.x], c1 = ctaCellPtr[blockIdx.x + 1];
    if (c0 < c1) {      // uniform over the CTA
        for (uint32_t k = c0; k < c1; ++k) stepCell<false>(cells[ctaCells[k]], nsteps, threadIdx.x, blockDim.x);
        return;
    }
    uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t lane = threadIdx.x & 31;
    if (w >= nWarps) return;
    for (uint32_t k = warpCellPtr[w]; k < warpCellPtr[w + 1]; ++k) {
        const DevCell& c = cells[warpCells[k]];
        stepCell<true>(c, nsteps, lane, 32);
    }
}

__device__ void reinitGatesCompt(const DevCell& c, uint32_t ic) {
    Row vRow = tableRow(c.V[ic], c.vMin, c.vMax, c.vDx, c.vCol);
    for (uint32_t q = c.chanPtr[ic]; q < c.chanPtr[ic + 1]; ++q) {
        int32_t s = c.stateOff[q];
        double C1, C2;
        if (c.Xpow[q] > 0.0) {
            tableLookup(c.vTab, c.vCol, c.colX[q], vRow, C1, C2);
            c.state[s++] = C1 / C2;
        }
        if (c.Ypow[q] > 0.0) {
            tableLookup(c.vTab, c.vCol, c.colY[q], vRow, C1, C2);
            c.state[s++] = C1 / C2;
        }
        if (c.Zpow[q] > 0.0) {
            int32_t src = c.zSrc[q];
            if (src >= 0) {
                Row r = tableRow(c.ca[src], c.caMin, c.caMax, c.caDx, c.caCol);
                tableLookup(c.caTab, c.caCol, c.colZ[q], r, C1, C2);
            } else if (c.extCa[q] > 0) {
                Row r = tableRow(c.extCa[q], c.caMin, c.caMax, c.caDx, c.caCol);
                tableLookup(c.caTab, c.caCol, c.colZ[q], r, C1, C2);
            } else {
                tableLookup(c.vTab, c.vCol, c.colZ[q], vRow, C1, C2);
            }
            c.state[s] = C1 / C2;
        }
    }
}

// HSolveActive::reinit (hsolve/HSolveActiveSetup.cpp:43-160) and the reinit
// of the tick-1/4 objects (SynChan::vReinit, SimpleSynHandler::vReinit with
// the description's events queued again, HHChannel2D X), one warp per cell.
__global__ void hsReinitFp64(const DevCell* __restrict__ cells, uint32_t nCells) {
    uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t lane = threadIdx.x & 31;
    if (w >= nCells) return;
    const DevCell& c = cells[w];
    for (uint32_t k = lane; k < c.S; k += 32) {
        c.synXc1[k] = c.synConst[5 * k];
        c.synXc2[k] = c.synConst[5 * k + 1];
        c.synYc1[k] = c.synConst[5 * k + 2];
        c.synYc2[k] = c.synConst[5 * k + 3];
        c.synNorm[k] = c.synConst[5 * k + 4];
        c.synX[k] = 0.0;
        c.synY[k] = 0.0;
        c.synAct[k] = 0.0;
        c.synGk[k] = 0.0;
        c.evCur[k] = c.evPtr[k];
    }
    for (uint32_t i = lane; i < c.N; i += 32) {
        c.V[i] = c.initVm[i];
        c.ext[2 * i] = 0.0;
        c.ext[2 * i + 1] = 0.0;
        c.injVarying[i] = 0.0;
    }
    for (uint32_t k = lane; k < c.SG; k += 32) c.sgLast[k] = -c.sgRefract[k];
    for (uint32_t p = lane; p < c.P; p += 32) {
        c.iCa[p] = 0.0;
        c.c[p] = 0.0;
        c.ca[p] = c.CaBasal[p];
    }
    if (lane == 0) {
        c.ctl->nSteps = 0;
        c.ctl->stimPtr = 0;
        c.ctl->nSpikes = 0;
        c.ctl->nSamples = 0;
        c.ctl->err = 0;
    }
    __syncwarp();
    // sendValues: the tick-4 objects see initVm and CaBasal
    // tick-1 objects reinit before the solver: their concentrations reach
    // the channels' external calcium the gates start from
    if (lane == 0 && c.nDif) difReinit(c);
    __syncwarp();
    for (uint32_t k = lane; k < c.K2; k += 32) {
        c.c2dX[k] = c.c2dX0[k];
        c.c2dGk[k] = 0.0;
        c.c2dVm[k] = c.V[c.c2dCompt[k]];
        c.c2dC1[k] = c.c2dConc1[k] >= 0 ? c.ca[c.c2dConc1[k]] : 0.0;
        c.c2dC2[k] = c.c2dConc2[k] >= 0 ? c.ca[c.c2dConc2[k]] : 0.0;
    }
    for (uint32_t ic = lane; ic < c.N; ic += 32) reinitGatesCompt(c, ic);
    // a Table reading Vm at reinit records sample 0
    if (c.nRec && c.recCap) {
        for (uint32_t r = lane; r < c.nRec; r += 32) c.recBuf[r] = recValue(c, c.recCompt[r]);
        __syncwarp();
        if (lane == 0) c.ctl->nSamples = 1;
    }
}

__global__ void hsScatterFields(const FieldWrite* __restrict__ w, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const FieldWrite x = w[i];
    if (x.size == 8) *static_cast<unsigned long long*>(x.addr) = x.bits;
    else if (x.size == 4) *static_cast<uint32_t*>(x.addr) = (uint32_t)x.bits;
    else *static_cast<uint8_t*>(x.addr) = (uint8_t)x.bits;
}

// Spike read-back of a batch: each cell's spike count, then every cell's
// stored spikes gathered into one list (cell c at off[c] .. off[c+1]), so
// that the host reads all cells with one copy per array.
__global__ void hsSpikeCountsFp64(const DevCell* __restrict__ cells, uint32_t nCells, uint32_t* __restrict__ counts) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < nCells) counts[c] = cells[c].ctl->nSpikes;
}

__global__ void hsGatherSpikesFp64(const DevCell* __restrict__ cells, uint32_t nCells,
                                   const uint32_t* __restrict__ off, uint32_t* __restrict__ gen,
                                   double* __restrict__ time) {
    const uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (c >= nCells) return;
    const uint32_t o = off[c], m = off[c + 1] - o;
    const DevCell& d = cells[c];
    for (uint32_t i = lane; i < m; i += 32) {
        gen[o + i] = d.spikeGen[i];
        time[o + i] = d.spikeTime[i];
    }
}

__global__ void hsGatherSpikesMixed(const uint32_t* __restrict__ srcGen, const float* __restrict__ srcTime,
                                    uint32_t cap, uint32_t nCells, const uint32_t* __restrict__ off,
                                    uint32_t* __restrict__ gen, double* __restrict__ time) {
    const uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (c >= nCells) return;
    const uint32_t o = off[c], m = off[c + 1] - o;
    for (uint32_t i = lane; i < m; i += 32) {
        gen[o + i] = srcGen[(size_t)c * cap + i];
        time[o + i] = (double)srcTime[(size_t)c * cap + i];
    }
}

// One value per entry of a gather list: out[k] = *src[k] (a double, or a
// float when f32), NaN for a null entry.
__global__ void hsGatherValues(const void* const* __restrict__ src, uint32_t f32, uint64_t n,
                               double* __restrict__ out) {
    const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const void* p = src[k];
    out[k] = !p ? __longlong_as_double(0x7FF8000000000000ll)
                : f32 ? (double)*static_cast<const float*>(p) : *static_cast<const double*>(p);
}

cudaError_t launchGatherValues(const void* const* src, uint32_t f32, uint64_t n, double* out, cudaStream_t st) {
    if (!n) return cudaSuccess;
    hsGatherValues<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(src, f32, n, out);
    return cudaGetLastError();
}

cudaError_t launchSpikeCountsFp64(const DevCell* cells, uint32_t nCells, uint32_t* counts, cudaStream_t st) {
    if (!nCells) return cudaSuccess;
    hsSpikeCountsFp64<<<(nCells + 255) / 256, 256, 0, st>>>(cells, nCells, counts);
    return cudaGetLastError();
}

cudaError_t launchGatherSpikes(const DevCell* cells, const uint32_t* srcGen, const float* srcTime, uint32_t cap,
                               uint32_t nCells, const uint32_t* off, uint32_t* gen, double* time,
                               cudaStream_t st) {
    if (!nCells) return cudaSuccess;
    const uint32_t blocks = (nCells * 32 + 255) / 256;
    if (cells) hsGatherSpikesFp64<<<blocks, 256, 0, st>>>(cells, nCells, off, gen, time);
    else hsGatherSpikesMixed<<<blocks, 256, 0, st>>>(srcGen, srcTime, cap, nCells, off, gen, time);
    return cudaGetLastError();
}

cudaError_t launchScatterFields(const FieldWrite* w, uint32_t n, cudaStream_t st) {
    if (!n) return cudaSuccess;
    hsScatterFields<<<(n + 255) / 256, 256, 0, st>>>(w, n);
    return cudaGetLastError();
}

cudaError_t launchStepFp64(const DevCell& c, uint32_t nsteps, cudaStream_t st) {
    hsStepFp64<<<1, 256, 0, st>>>(c, nsteps);
    return cudaGetLastError();
}

cudaError_t launchStepFp64Cluster(const DevCell& c, uint32_t ctas, uint32_t nsteps, cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = ctas;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(ctas);
    cfg.blockDim = dim3(256);
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, hsStepFp64Cluster, c, nsteps);
}

// `ctas` CTAs per solver: 1 = one CTA each (no cluster), 2..8 = a cluster each
cudaError_t launchGroupStepFp64(const DevCell* cells, uint32_t n, uint32_t ctas, uint32_t nsteps,
                                cudaStream_t st) {
    if (!n) return cudaSuccess;
    if (ctas <= 1) {
        hsGroupStepFp64<<<n, 256, 0, st>>>(cells, nsteps);
        return cudaGetLastError();
    }
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = ctas;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(n * ctas);
    cfg.blockDim = dim3(256);
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, hsGroupStepFp64Cluster, cells, nsteps);
}

cudaError_t launchBatchStepFp64(const DevCell* cells, const uint32_t* warpCellPtr,
                                const uint32_t* warpCells, uint32_t nWarps, const uint32_t* ctaCellPtr,
                                const uint32_t* ctaCells, uint32_t nsteps, uint32_t threadsPerCta,
                                cudaStream_t st) {
    uint32_t blocks = (nWarps * 32 + threadsPerCta - 1) / threadsPerCta;
    hsBatchStepFp64<<<blocks, threadsPerCta, 0, st>>>(cells, warpCellPtr, warpCells, nWarps, ctaCellPtr, ctaCells,
                                                      nsteps);
    return cudaGetLastError();
}

int fp64BatchCtasPerSm(uint32_t threadsPerCta) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, hsBatchStepFp64, (int)threadsPerCta, 0) != cudaSuccess)
        return 0;
    return n;
}

cudaError_t launchReinitFp64(const DevCell* cells, uint32_t nCells, cudaStream_t st) {
    uint32_t blocks = (nCells * 32 + 255) / 256;
    hsReinitFp64<<<blocks ? blocks : 1, 256, 0, st>>>(cells, nCells);
    return cudaGetLastError();
}

}  // namespace hsg
