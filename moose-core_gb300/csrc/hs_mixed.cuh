// hs_mixed.cuh -- device layout of the mixed-precision batched HSolve.
//
// Matrix.  Each cell's compartments are nodes of a tree rooted at the
// morphological root; every junction of three or more compartments (a
// `coupled_` group of hsolve/HinesMatrix.cpp:84-130) becomes one extra node
// without membrane: the reference's clique of conductances Ga_i*Ga_j/sum(Ga)
// between the members is exactly the star with conductance Ga_i from each
// member to that node, once the node is eliminated (Y-Delta transform), so the
// voltages are the same.  The matrix is then a plain tree: each node has one
// coupling (off) to its parent.
//
// Forests.  Cells are grouped into forests that one CTA steps together.  A
// forest's nodes are numbered level-major: level 0 holds the roots of all its
// cells, level d+1 the children of level d, the children of one node
// contiguous and junction nodes after compartments.  A level is one parallel
// step of the elimination, so narrow levels of one cell fill up with the
// levels of the others.  During elimination a forest keeps its pivots, right
// hand sides and coupling topology in shared memory when it fits ("shared
// forest"); otherwise in global scratch ("global forest").
//
// Per-node arrays: structure of arrays over all nodes (forest after forest),
// with fixed "slots" so that a warp's loads are coalesced:
//   channel slot j (< kMaxChan): type byte j of ctype4[n], gbar[j*ld + n]
//   gate state of channel j, gate g (X,Y,Z): state[(3*j+g)*ld + n]
//   at most one Ca pool, one HHChannel2D per compartment; SynChans in CSR.
//
// Precision: rate tables, gate increments, channel conductances, K(Ca), Ca
// pools and synapses are FP32; gate states are two-float sums (~48 bits)
// that accumulate the FP32 increments; Vm, matrix assembly, forward
// elimination and back substitution are FP64.
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
// bits 16..27: gate present, bit kNodeGateShift + 3*slot + gate (X, Y, Z)
constexpr uint32_t kNodeGateShift = 16;

// One HHChannel prototype (hsolve/HSolveStruct.h:55-108), 16 bytes so that
// a kernel reads it with one vector load; general (non-integer) powers are
// in a separate table.
struct alignas(16) ChanType {
    float ek;
    int8_t xp, yp, zp;     // powers 1..4, -1 general (the type's ChanPow), 0 absent
    int8_t instant;
    int16_t colX, colY, colZ;   // table columns (floats) of A for X/Y/Z
    int8_t zCa;            // 1: Z gate on the Ca table with the node's pool
    int8_t caTarget;       // 1: feeds the node's pool
};
static_assert(sizeof(ChanType) == 16, "ChanType is one 16-byte load");

struct ChanPow {           // general powers of a channel type's X, Y, Z
    float x, y, z, pad;
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

constexpr uint32_t kNoParent = 0xFFFF;   // MixBatch::par of a root
constexpr uint32_t kMaxForestNodes = 0xFFFF;
constexpr uint32_t kSmemLevels = 1024;      // level offsets kept in shared memory
constexpr uint32_t kWsLevels = 256;         // per-level counters of the split step

// A forest: nodes [node0, node0 + nNodes), level offsets (forest-local)
// levelPtr[level0 .. level0 + nLevels], cells forestCells[cell0 ..].
struct MixForest {
    uint32_t node0, nNodes;
    uint32_t level0, nLevels;
    uint32_t cell0, nCells;
    uint32_t shared;             // 1: elimination arrays staged in shared memory
    uint32_t pad;
};

// Per-cell entries of the inject, stimulus, SpikeGen and recording lists.
struct MixCellRange {
    uint32_t inj0, nInj;         // inject entries (injVal)
    uint32_t stim0, nStim;       // stimulus schedule entries
    uint32_t sg0, nSg;           // SpikeGens
    uint32_t rec0, nRec;         // recorded nodes (columns rec0..)
};

// A per-node array prefetched into L2 ahead of the assembly: `n` elements
// of `elem` bytes from `base`, node k at base + k * elem.
constexpr int kMaxPrefetch = 32;
struct PrefetchArr {
    const void* base;
    uint32_t elem;
    uint32_t n;
};

// One value written into device memory by hsScatterValues: the float
// (f32 = 1) or double (f32 = 0) at `addr`.
struct ValueWrite {
    void* addr;
    double value;
    uint32_t f32;
    uint32_t pad;
};

struct MixBatch {
    uint32_t nCells;
    // prototypes of this batch (read-only device tables)
    const ChanType* chanTypes;
    const ChanPow* chanPow;
    const C2dType* c2dTypes;
    const SynType* synTypes;     // at the clock dt, written by reinit
    uint64_t ld;                 // slot stride (number of nodes, padded)
    float dtf;
    double dt;
    int caAdvance;
    uint32_t nForests;
    const MixCellRange* cells;
    const MixForest* forests;
    unsigned long long* forestStep;      // steps done by each forest
    const unsigned long long* stopStep;  // per cell: no step at or after this one
    const unsigned long long* forestStop;   // per forest: the largest stop step of its cells
    uint32_t anyStop;                    // 0: no cell has a stop step
    const uint32_t* cellOf;              // per node: its cell
    const uint32_t* forestCells;
    const uint32_t* levelPtr;
    // per node (global index)
    const uint32_t* nodeInfo;    // flags, K(Ca) type, gate mask (bits above)
    const uint32_t* ctype4;      // 4 channel type bytes
    const uint32_t* topo;        // forest-local first child | child count << 16 | level (<= 255) << 24
    const uint16_t* par;         // forest-local parent, kNoParent for a root
    uint32_t* err;               // set to 1 when a bounded wait gave up
    uint32_t waitRounds;         // sleep rounds of one bounded wait
    const uint32_t* injIdx;      // inject entry of a kNodeInject node
    const double *off, *HS2, *CmByDt, *EmByRm;
    double* V;
    double *elimD, *elimR;       // elimination scratch of global forests
    float *caG, *caGE;           // Ca-feeding conductance of the step
    const float* gbar;           // [kMaxChan][ld]  Gbar * modulation
    float2* state;               // [3*kMaxChan][ld] gate states, two-float sums hi + lo
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
    float2* synGk;               // Gk, Gk*Ek of the step the assembly adds next
    const uint32_t* synCell;     // cell of each SynChan
    uint32_t* evCur;
    const uint32_t* evEnd;
    const uint32_t* evStep;      // delivery step of each event
    const float* evAct;          // weight / dt
    // inject / stimulus
    double* injVal;
    const uint32_t *stimStep, *stimEntry;
    const double* stimValue;
    uint32_t* stimCur;
    // spike gens
    const uint32_t* sgNode;      // global node
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
    const uint32_t* recNode;     // global node of each column
    double* recBuf;
    uint32_t recLd, recCap, recStride;
    unsigned long long* stepCount;
    // arrays the assembly reads per node (L2 prefetch)
    PrefetchArr pf[kMaxPrefetch];
    uint32_t nPf;
};

}  // namespace hsg
