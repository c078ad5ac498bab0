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
// Layout: structure of arrays indexed by node, with fixed "slots" so that all
// of a node's loads are independent and coalesced across the lanes of a warp:
//   channel slot j (< kMaxChan): type byte j of ctype4[n], gbar[j*ld + n]
//   gate state of channel j, gate g (X,Y,Z): state[(3*j+g)*ld + n]
//   at most one Ca pool, one HHChannel2D per compartment; SynChans in CSR.
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
constexpr int kMaxChan = 4;            // channel slots per compartment
constexpr uint8_t kNoType = 0xFF;

// bits of MixBatch::nodeInfo
constexpr uint32_t kNodeCenter = 1u << 0;    // junction node, no membrane
constexpr uint32_t kNodeInject = 1u << 1;    // has an inject entry
constexpr uint32_t kNodePool = 1u << 2;      // has a Ca pool
constexpr uint32_t kNodeSyn = 1u << 3;       // has SynChans
// bits 8..15: HHChannel2D type (kNoType: none)

struct ChanType {          // one HHChannel prototype (hsolve/HSolveStruct.h:55-108)
    float ek;
    int8_t xp, yp, zp;     // powers 1..4, -1 general (powf), 0 absent
    int8_t instant;
    float xpf, ypf, zpf;   // general powers
    int16_t colX, colY, colZ;   // table columns (floats) of A for X/Y/Z
    int8_t zCa;            // 1: Z gate on the Ca table with the node's pool
    int8_t caTarget;       // 1: feeds the node's pool
};

struct C2dType {           // one HHChannel2D prototype
    float ek;
    int8_t xp;             // power 1..4, -1 general
    int8_t dep0, dep1;     // 0 Vm, 1 conc (the node's pool), -1 none
    int8_t instant;
    int8_t gate;           // 2-D table
    int8_t pad[3];
    float xpf;
};

struct SynType {           // SynChan constants at the clock dt
    float xc1, xc2, yc1, yc2, ek;
};

// Elimination schedule of a cell: its nodes are numbered unit by unit.  A
// unit is eliminated serially by one thread: a whole small subtree in
// post-order (level 0) or an unbranched chain of the tree above those
// subtrees, bottom to top (levels >= 1).  Units of one level are independent;
// a unit's children lie in lower levels or earlier in the same unit.
struct MixCellRange {
    uint32_t node0, nNodes;      // global first node, count
    uint32_t level0, nLevels;    // offset into unitPtr (nLevels+1 entries)
    uint32_t unit0;              // offset into units
    uint32_t child0;             // offset into childList
    uint32_t inj0, nInj;         // inject entries
    uint32_t stim0, nStim;       // stimulus schedule entries
    uint32_t sg0, nSg;           // SpikeGens
    uint32_t rec0, nRec;         // recorded nodes (columns rec0..)
};

struct MixBatch {
    uint32_t nCells;
    uint64_t ld;                 // slot stride (number of nodes, padded)
    float dtf;
    double dt;
    int caAdvance;
    const MixCellRange* cells;
    const uint32_t* unitPtr;     // cell-local unit offsets per level
    const uint2* units;          // cell-local node range [x, y) of each unit
    const uint32_t* childList;   // cell-local children, per cell from child0
    // per node (global index)
    const uint32_t* nodeInfo;    // flags; bits 8-15 K(Ca) type; bits 16-23 child count
    const uint32_t* ctype4;      // 4 channel type bytes
    const uint32_t* childStart;  // into the cell's childList
    const uint32_t* parent;      // cell-local node index, ~0u for the root
    const double *off, *offsq, *HS2, *CmByDt, *EmByRm;
    double* V;
    double *inv, *gEl, *VMid;    // elimination temporaries
    float *caG, *caGE;           // Ca-feeding conductance of the step
    const float* gbar;           // [kMaxChan][ld]  Gbar * modulation
    float* state;                // [3*kMaxChan][ld]
    float* chanGk;               // [kMaxChan][ld] last conductance
    // pool (one per node)
    float *poolC, *poolCa;
    const float *poolG1, *poolF2, *poolBasal, *poolCeil, *poolFloor;   // poolG1 = 1 - factor1
    // HHChannel2D (one per node)
    const float* k2gbar;         // Gbar * modulation
    float* k2x;
    const float* g2d;            // interleaved (A,B) tables, FP32
    const uint64_t* g2dOff;
    const float* g2dGeom;        // xmin, ymin, invDx, invDy, xmax, ymax per table
    const uint32_t* g2dN;        // nx, ny
    // SynChans
    const uint32_t* syn0;        // CSR (ld+1)
    const uint8_t* synType;
    const float* synNorm;        // norm * modulation
    float *synX, *synY;
    uint32_t* evCur;
    const uint32_t* evEnd;
    const uint32_t* evStep;      // delivery step of each event
    const float* evAct;          // weight / dt
    // inject / stimulus
    const uint32_t* injNode;
    double* injVal;
    const uint32_t *stimStep, *stimEntry;
    const double* stimValue;
    uint32_t* stimCur;
    // spike gens
    const uint32_t* sgNode;
    const float *sgThresh, *sgRefract;
    const int32_t* sgEdge;
    float* sgLast;
    int32_t* sgFired;
    uint32_t spikeCap;
    uint32_t* spikeCount;
    uint32_t* spikeGen;
    float* spikeTime;
    // rate tables (FP32), A/B interleaved per species
    const float* vTab;
    uint32_t vCol, vRows;
    float vMin, vMax, vInvDx;
    const float* caTab;
    uint32_t caCol, caRows;
    float caMin, caMax, caInvDx;
    // recording
    const uint32_t* recNode;
    double* recBuf;
    uint32_t recLd, recCap, recStride;
    unsigned long long* stepCount;
};

}  // namespace hsg
