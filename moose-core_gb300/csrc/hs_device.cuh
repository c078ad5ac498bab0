// hs_device.cuh -- device layout of one HSolve cell and the per-step device
// functions shared by the GB300 kernels.
//
// Every array is structure-of-arrays in Hines order.  The FP64 functions here
// keep the reference's operation order exactly (compile with --fmad=false):
//   rate lookup          hsolve/RateLookup.cpp:62-103
//   gate update          hsolve/HSolveActive.cpp:218-332 (trapezoidal)
//   channel conductance  hsolve/HSolveStruct.cpp:53-65
//   matrix row update    hsolve/HSolveActive.cpp:85-151
//   elimination          hsolve/HSolvePassive.cpp:246-401 (as pull programs)
//   calcium              hsolve/HSolveActive.cpp:153-216, HSolveStruct.cpp:139-155
//   HHChannel2D          biophysics/HHChannel2D.cpp:327-369, builtins/Interpol2D.cpp:508-592
//   SynChan              biophysics/SynChan.cpp:200-224, synapse/SimpleSynHandler.cpp:98-113
//   SpikeGen             biophysics/SpikeGen.cpp:202-216
#pragma once

#include <cstdint>

namespace hsg {

constexpr uint32_t kDifState = 13;

// A recording entry: the value's index in its array (bits 0-27) and what is
// recorded (bits 28-31): the compartment's Vm (VmOut), the channel's Ik =
// (Ek - Vm) Gk as HSolveActive::sendValues sends it (IkOut), the channel's
// Gk, or the pool's Ca (concOut).
constexpr uint32_t kRecShift = 28;
constexpr uint32_t kRecVm = 0, kRecIk = 1, kRecGk = 2, kRecCa = 3;

struct DevCtl {
    unsigned long long nSteps;   // steps since reinit
    uint32_t stimPtr;
    uint32_t nSpikes;            // spikes produced (may exceed capacity)
    uint32_t nSamples;           // trace samples produced
    uint32_t err;
};

struct DevCell {
    uint32_t N, H, C, G, P, K2, S, SG, nStim;
    uint32_t fLevels, bLevels;
    uint32_t fWaves;             // forward sweep as waves (0: level programs)
    int caAdvance;
    double dt;                   // clock dt
    // compartments
    double *V, *VMid, *M, *HJ0, *HS2, *CmByDt, *EmByRm, *injBasal, *injVarying, *ext, *prevExt;
    double* initVm;              // reinit values (HSolveActive::reinitCompartments)
    const uint32_t *chanPtr, *poolPtr, *extPtr;
    const int32_t* extList;
    // elimination programs
    const uint32_t *fLevelPtr, *fRows, *fOpPtr;
    const int4* fOps;
    const uint32_t *bLevelPtr, *bRows, *bTermPtr;
    const int2* bTerms;
    const uint32_t *fRun, *fRunRow, *bRun, *bRunRow;   // cable runs per level
    const uint32_t* fWavePtr;
    const int4* fWaveOps;        // per fused update: {t1, a1, t2, a2}, {l, p, -, -}
    // channels
    double *Gbar, *Ek, *Xpow, *Ypow, *Zpow, *mod, *Gk, *state, *extCa;
    int32_t* instant;
    const int32_t *stateOff, *colX, *colY, *colZ, *zSrc;
    const uint32_t* chanCompt;
    // pools
    double *c, *CaBasal, *f1, *f2, *ceil, *floor_, *ca, *iCa;
    const uint32_t *feedPtr, *feedChan;
    // rate tables
    const double* vTab;
    uint32_t vCol;
    double vMin, vMax, vDx;
    const double* caTab;
    uint32_t caCol;
    double caMin, caMax, caDx;
    // HHChannel2D
    const double* g2dAB;
    const uint64_t* g2dOff;          // per gate2d: offset (in doubles) into g2dAB
    const double* g2dGeom;           // per gate2d: xmin,xmax,ymin,ymax,invDx,invDy
    const uint32_t* g2dN;            // per gate2d: nx, ny
    const uint32_t* c2dCompt;
    const int32_t *c2dGate, *c2dDep0, *c2dDep1, *c2dConc1, *c2dConc2, *c2dInstant;
    double *c2dGbar, *c2dEk, *c2dXpow, *c2dMod, *c2dX, *c2dGk, *c2dVm, *c2dC1, *c2dC2;
    const double* c2dX0;         // X at reinit
    // SynChans
    const uint32_t* synCompt;
    double *synEk, *synMod, *synX, *synY, *synAct, *synGk, *synXc1, *synXc2, *synYc1, *synYc2, *synNorm;
    const double* synConst;      // per SynChan: xc1, xc2, yc1, yc2, norm at the clock dt
    const uint32_t* evPtr;
    uint32_t* evCur;
    const double *evTime, *evW;
    // SpikeGens
    const uint32_t* sgCompt;
    double *sgThreshold, *sgRefract, *sgLast;
    int32_t *sgEdge, *sgFired;
    uint32_t spikeCap;
    uint32_t* spikeGen;
    double* spikeTime;
    // stimulus
    const uint32_t *stimStep, *stimCompt;
    const double* stimValue;
    uint8_t* injPresent;
    // tick-1 external calcium: objects, messages, state (kDifState x nDif:
    // C, prevC, dCbyDt, Cmultiplier, bFree, bBound, prevFree, Af, Bf,
    // activation, volume, outerArea, innerArea)
    uint32_t nDif;
    const int32_t* difKind;
    const double* difPar;
    const uint32_t *difOff, *difDst, *ikOff, *ikDst;
    double* difState;
    // trace recording
    uint32_t nRec, recStride, recCap, recLd;
    const uint32_t* recCompt;
    double* recBuf;
    DevCtl* ctl;
};

// One queued field write of the drop-in: `size` (1, 4 or 8) bytes of `bits`
// to `addr`, an address inside the solver's arena aligned to `size`.
struct FieldWrite {
    void* addr;
    unsigned long long bits;
    uint32_t size;
    uint32_t pad;
};

// The value a recording entry names (hsolve/HSolveActive.cpp:354-385 for Ik).
__device__ __forceinline__ double recValue(const DevCell& c, uint32_t e) {
    const uint32_t i = e & ((1u << kRecShift) - 1);
    switch (e >> kRecShift) {
    case kRecIk: return (c.Ek[i] - c.V[c.chanCompt[i]]) * c.Gk[i];
    case kRecGk: return c.Gk[i];
    case kRecCa: return c.ca[i];
    default: return c.V[i];
    }
}

// ---------------------------------------------------------------------------
// FP64 helpers, reference order

struct Row {
    int64_t off;      // first column of the row
    double frac;
};

__device__ __forceinline__ Row tableRow(double x, double mn, double mx, double dx, uint32_t nCol) {
    if (x < mn) x = mn;
    else if (x > mx) x = mx;
    double div = (x - mn) / dx;
    unsigned int integer = (unsigned int)(div);
    Row r;
    r.frac = div - integer;
    r.off = (int64_t)integer * nCol;
    return r;
}

__device__ __forceinline__ void tableLookup(const double* T, uint32_t nCol, int32_t column,
                                            const Row& r, double& C1, double& C2) {
    const double* ap = T + r.off + column;
    const double* bp = ap + nCol;
    double a = ap[0], b = bp[0];
    C1 = a + (b - a) * r.frac;
    a = ap[1];
    b = bp[1];
    C2 = a + (b - a) * r.frac;
}

__device__ __forceinline__ double gateStep(double x, double C1, double C2, double dt, bool inst) {
    if (inst) return C1 / C2;
    double temp = 1.0 + dt / 2.0 * C2;
    return (x * (2.0 - temp) + dt * C1) / temp;
}

__device__ __forceinline__ double takePower(double x, double p) {
    if (p == 1.0) return x;
    if (p == 2.0) return x * x;
    if (p == 3.0) return x * x * x;
    if (p == 4.0) {
        double y = x * x;
        return y * y;
    }
    if (x > 0.0) return exp(p * log(x));
    return 0.0;
}

// Interpol2D::innerLookup + interpolate on interleaved (A,B) pairs.
__device__ __forceinline__ void interp2dBoth(const double* AB, const double* geom, uint32_t nx,
                                             uint32_t ny, double x, double y, double& A,
                                             double& B) {
    double xmin = geom[0], xmax = geom[1], ymin = geom[2], ymax = geom[3];
    if (x < xmin) x = xmin;
    if (x > xmax) x = xmax;
    if (y < ymin) y = ymin;
    if (y > ymax) y = ymax;
    double xv = (x - xmin) * geom[4];
    unsigned long xi = (unsigned long)xv;
    if (xi >= nx) xi = nx - 1;
    bool endX = xi == nx - 1;
    double xF = xv - xi;
    double yv = (y - ymin) * geom[5];
    unsigned long yi = (unsigned long)yv;
    if (yi >= ny) yi = ny - 1;
    bool endY = yi == ny - 1;
    double yF = yv - yi;
    double xFyF = xF * yF;
    const double* p00 = AB + 2 * (xi * ny + yi);
    double a00 = p00[0], b00 = p00[1];
    double a01 = 0.0, b01 = 0.0, a10 = 0.0, b10 = 0.0, a11 = 0.0, b11 = 0.0;
    if (!endX) {
        const double* p10 = p00 + 2 * ny;
        a10 = p10[0]; b10 = p10[1];
        if (!endY) {
            a11 = p10[2]; b11 = p10[3];
            a01 = p00[2]; b01 = p00[3];
        }
    } else if (!endY) {
        a01 = p00[2]; b01 = p00[3];
    }
    double w00 = 1 - xF - yF + xFyF, w10 = xF - xFyF, w01 = yF - xFyF;
    A = a00 * w00 + a10 * w10 + a01 * w01 + a11 * xFyF;
    B = b00 * w00 + b10 * w10 + b01 * w01 + b11 * xFyF;
}

}  // namespace hsg
