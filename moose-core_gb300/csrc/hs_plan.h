// hs_plan.h -- host-side HSolve setup for the GB300 solver.
//
// Builds, from an HsCellDesc, everything `HSolveActive::setup` builds
// (hsolve/HSolveActiveSetup.cpp:17-41): the Hines ordering of
// `HSolvePassive::walkTree` (hsolve/HSolvePassive.cpp:45-98), the matrix and
// junction groups of `HinesMatrix::setup` (hsolve/HinesMatrix.cpp:25-223),
// channel/gate/Ca-pool arrays and the merged rate tables of
// `createLookupTables` (hsolve/HSolveActiveSetup.cpp:339-526).
//
// The reference walks its elimination as one serial sweep over an operand
// "pointer program" (`makeOperands`, hsolve/HinesMatrix.cpp:226-365).  Here
// that program is recompiled into a *pull* form: every matrix entry belongs
// to one row, each row applies the updates aimed at its entries in the
// reference's order, and rows are grouped into dependency levels.  All rows
// of a level can run in parallel and the result is bit-identical to the
// serial sweep, because each entry still sees the same operations in the
// same order.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/moose_gb300.h"

namespace hsg {

// One forward-elimination update `t -= (l / diag[p]) * a` (entries index the
// cell's M array: [0,N) diag, [N,2N) rhs, [2N,2N+H) HJ, [2N+H,3N+H) off).
struct FwdOp {
    int32_t t, l, a, p;
};
// Two forward updates that share one quotient: M[t1] -= q * M[a1], then
// M[t2] -= q * M[a2] (t2 < 0: none), q = M[l] / M[p].
struct FwdPair {
    int32_t t1, a1, t2, a2, l, p, pad0, pad1;
};
// One back-substitution term `v -= coef * VMid[src]`.
struct BwdTerm {
    int32_t coef, src;
};

struct Table {
    double min = 0, max = 0, dx = 0;
    uint32_t nPts = 0, nCol = 0;
    std::vector<double> data;  // nPts x nCol, row-major, [A,B] per species
};

struct Gate2D {
    double xmin, xmax, ymin, ymax, invDx, invDy;
    uint32_t nx, ny;           // xdivs+1, ydivs+1
    const double *srcA, *srcB; // the description's tables (identity for sharing)
    std::vector<double> AB;    // interleaved A,B: [(ix*ny+iy)*2 + {0,1}] (if copied)
};

struct PlanOptions {
    bool copyTables2d = true;  // batches share 2-D tables and skip the copy
};

struct CellPlan {
    uint32_t N = 0, H = 0;
    double dtSetup = 0;
    std::vector<uint32_t> modelOf;      // hines -> model compartment
    std::vector<int64_t> hinesOf;       // model -> hines (-1 if not in tree)
    // compartments (Hines order)
    std::vector<double> V0, initVm, CmByDt, EmByRm, HS2, off, injBasal;
    std::vector<uint8_t> injPresent;
    std::vector<double> Ra, Rm, Cm, Em;
    std::vector<std::vector<uint32_t>> children;
    std::vector<double> HJ0;            // HJCopy
    // elimination programs
    std::vector<uint32_t> fLevelPtr, fRows, fOpPtr;   // fOpPtr indexed by position in fRows
    std::vector<FwdOp> fOps;
    std::vector<uint32_t> bLevelPtr, bRows, bTermPtr;
    std::vector<BwdTerm> bTerms;
    // Cable runs: at the first level of a run of consecutive one-row levels
    // whose rows are plain cable rows (forward: rows r0, r0+1, ... each
    // updated only by the previous row; backward: rows i0, i0-1, ... each
    // with the single term on the next row), the run's length and first
    // row; 0 elsewhere.  Per level.
    std::vector<uint32_t> fRun, fRunRow, bRun, bRunRow;
    uint32_t maxLevelWidthF = 0, maxLevelWidthB = 0;
    // The forward sweep as waves (empty: the level programs are used).  The
    // updates of the level programs, in their order, with each pair that
    // shares a quotient fused, are placed in the earliest wave after every
    // update they depend on: after the last write of each entry they read
    // or write, and after the last read of each entry they write.  The
    // updates of a wave touch disjoint entries, so a wave runs in any order
    // or all at once, and each entry sees the updates of the level programs
    // in their order: the same operations on the same values.
    std::vector<uint32_t> fWavePtr;
    std::vector<FwdPair> fWaveOps;
    // channels (solver order)
    uint32_t C = 0, G = 0;
    std::vector<uint32_t> chanPtr;      // N+1
    std::vector<double> Gbar, Ek, Xpow, Ypow, Zpow, modulation;
    std::vector<int32_t> instant, stateOff, colX, colY, colZ, zSrc;  // zSrc: pool, -1 V row, -2 extCa row
    std::vector<uint32_t> chanModel;
    std::vector<int64_t> chanSolverOf;  // model -> solver
    std::vector<double> state0;
    // pools (solver order)
    uint32_t P = 0;
    std::vector<uint32_t> poolPtr;      // N+1 pools of each compartment
    std::vector<double> CaBasal, f1, f2, ceiling, floor_, c0;
    std::vector<int32_t> caTarget;      // per channel: pool or -1
    std::vector<uint32_t> feedPtr, feedChan;  // per pool: channels feeding it, channel order
    std::vector<uint32_t> poolModel;
    std::vector<int64_t> poolSolverOf;
    Table vTable, caTable;
    double vMin = 0, vMax = 0, caMin = 0, caMax = 0;
    int vDiv = 0, caDiv = 0;
    // external tick-4 objects
    uint32_t K2 = 0, S = 0, SG = 0;
    std::vector<Gate2D> gates2d;
    std::vector<uint32_t> c2dCompt;     // hines
    std::vector<double> c2dGbar, c2dEk, c2dXpow, c2dMod, c2dX0;
    std::vector<int32_t> c2dGate, c2dDep0, c2dDep1, c2dConc1, c2dConc2, c2dInstant;
    std::vector<uint32_t> synCompt;     // hines
    std::vector<double> synGbar, synEk, synTau1, synTau2, synMod;
    std::vector<uint32_t> evPtr;        // S+1
    std::vector<double> evTime, evW;
    // per compartment, external channels in tick-4 send order:
    // code >= 0: HHChannel2D k; code < 0: SynChan (-code - 1)
    std::vector<uint32_t> extPtr;
    std::vector<int32_t> extList;
    std::vector<uint32_t> sgCompt;
    std::vector<double> sgThreshold, sgRefract;
    std::vector<int32_t> sgEdge;
    std::vector<uint32_t> stimStep, stimCompt;
    std::vector<double> stimValue;
    // tick-1 external calcium (DifShell, DifBuffer, MMPump) in process order;
    // messages CSR by (object, kind) for kinds HS_DMSG_OUTER .. HS_DMSG_PUMP,
    // in description order, HHChannel targets as solver channels; the
    // solver's IkOut sends CSR by solver channel
    uint32_t nDif = 0;
    std::vector<int32_t> difKind;
    std::vector<double> difPar;             // nDif x HS_DIF_NPAR
    std::vector<uint32_t> difOff, difDst;   // nDif * kDifMsgKinds + 1
    std::vector<uint32_t> ikOff, ikDst;     // C + 1
};

constexpr uint32_t kDifMsgKinds = 6;        // HS_DMSG_OUTER .. HS_DMSG_PUMP

// Build the plan; returns false and sets err on invalid input.
bool buildPlan(const HsCellDesc& d, uint32_t seed, double dt, CellPlan& plan, std::string& err,
               const PlanOptions& opt = PlanOptions());

// SynChan reinit constants (biophysics/SynChan.cpp:171-251), host libm.
void synchanConstants(double tau1, double tau2, double gbar, double dt, double* xc1,
                      double* xc2, double* yc1, double* yc2, double* norm);

}  // namespace hsg
