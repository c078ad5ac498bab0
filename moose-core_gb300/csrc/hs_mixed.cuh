// hs_mixed.cuh -- device layout of the mixed-precision batched HSolve.
//
// All cells of a batch are concatenated.  Each cell's compartments are nodes
// of a tree in breadth-first order from the morphological root; every
// junction of three or more compartments (a `coupled_` group of
// hsolve/HinesMatrix.cpp:84-130) becomes one extra node without membrane: the
// reference's clique of conductances Ga_i*Ga_j/sum(Ga) between the members is
// exactly the star with conductance Ga_i from each member to that node, once
// the node is eliminated (Y-Delta transform), so the voltages are the same.
// The matrix is then a plain tree: each node has one coupling to its parent.
//
// Precision: gate states, rate tables, channel conductances, K(Ca), Ca pools
// and synapses are FP32; Vm, matrix assembly, forward elimination and back
// substitution are FP64.
#pragma once

#include <cstdint>

namespace hsg {

constexpr int kMaxChanTypes = 64;
constexpr int kMaxC2dTypes = 16;
constexpr int kMaxSynTypes = 16;

// bits of MixBatch::nodeInfo
constexpr uint32_t kNodeCenter = 1u << 0;    // junction node, no membrane
constexpr uint32_t kNodeInject = 1u << 1;    // has a basal/varying inject entry

struct ChanType {          // one HHChannel prototype (hsolve/HSolveStruct.h:55-108)
    float ek;
    int8_t xp, yp, zp;     // powers 1..4, -1 general (powf), 0 absent
    int8_t instant;
    float xpf, ypf, zpf;   // general powers
    int16_t colX, colY, colZ;   // table columns (floats) of A for X/Y/Z
    int8_t zSrc;           // -1: V table, >= 0: Ca table on the node's pool zSrc
    int8_t caTarget;       // pool (node-local) fed by this channel, or -1
};

struct C2dType {           // one HHChannel2D prototype
    float ek;
    int8_t xp;             // power 1..4, -1 general
    int8_t dep0, dep1;     // 0 Vm, 1 conc1, 2 conc2, -1 none
    int8_t conc1, conc2;   // node-local pools, or -1
    int8_t instant;
    int8_t gate;           // 2-D table
    float xpf;
};

struct SynType {           // SynChan constants at the clock dt
    float xc1, xc2, yc1, yc2, ek;
};

struct MixCellRange {
    uint32_t node0, nNodes;      // global first node, count
    uint32_t level0, nLevels;    // offset into levelPtr (nLevels+1 entries)
    uint32_t inj0, nInj;         // inject entries
    uint32_t stim0, nStim;       // stimulus schedule entries
    uint32_t sg0, nSg;           // SpikeGens
    uint32_t rec0, nRec;         // recorded nodes (columns rec0..)
};

struct MixBatch {
    uint32_t nCells;
    float dtf;
    double dt;
    int caAdvance;
    const MixCellRange* cells;
    const uint32_t* levelPtr;    // cell-local node offsets per level
    // per node (global index)
    const uint32_t* nodeInfo;
    const uint32_t* child0;      // CSR over children (global node indices)
    const uint32_t* parent;      // global node index, ~0u for the root
    const double *off, *HS2, *CmByDt, *EmByRm;
    double *V, *VMid, *rhsF, *inv;
    const uint32_t *chan0, *state0, *pool0, *c2d0, *syn0;   // CSR starts (n+1 entries)
    // channels
    const uint8_t* chanType;
    const float* chanGbar;       // Gbar * modulation
    float* state;
    float* chanGk;               // last conductance (field read-back)
    // pools
    float *poolC, *poolCa, *caG, *caGE;
    const float *poolF1, *poolF2, *poolBasal, *poolCeil, *poolFloor;   // poolF1 holds 1 - factor1
    // HHChannel2D
    const uint8_t* c2dType;
    const float* c2dGbar;        // Gbar * modulation
    float* c2dX;
    const float* g2d;            // interleaved (A,B) tables, FP32
    const uint64_t* g2dOff;
    const float* g2dGeom;        // xmin, ymin, invDx, invDy, xmax, ymax per table
    const uint32_t* g2dN;        // nx, ny
    // SynChans
    const uint8_t* synType;
    const float* synNorm;        // norm * modulation
    float *synX, *synY;
    uint32_t* evCur;
    const uint32_t* evEnd;       // per SynChan: end of its events
    const uint32_t* evStep;      // delivery step of each event
    const float* evAct;          // weight / dt
    // inject / stimulus
    const uint32_t* injNode;
    double* injVal;              // basal + varying per inject entry
    const uint32_t *stimStep, *stimEntry;
    const double* stimValue;
    uint32_t* stimCur;           // per cell
    // spike gens
    const uint32_t* sgNode;
    const float *sgThresh, *sgRefract;
    const int32_t* sgEdge;
    float* sgLast;
    int32_t* sgFired;
    uint32_t spikeCap;           // per cell
    uint32_t* spikeCount;        // per cell
    uint32_t* spikeGen;
    float* spikeTime;
    // rate tables (FP32): V table A/B interleaved per species
    const float* vTab;
    uint32_t vCol, vRows;        // rows = divisions + 2 (last row repeated)
    float vMin, vMax, vInvDx;
    const float* caTab;
    uint32_t caCol, caRows;
    float caMin, caMax, caInvDx;
    // recording
    const uint32_t* recNode;
    double* recBuf;
    uint32_t recLd, recCap, recStride;
    uint32_t* recCount;          // one counter for the batch
    unsigned long long* stepCount;   // per cell
};

}  // namespace hsg
