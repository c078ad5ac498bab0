/*
 * hsolve_oracle.c -- CPU restatement of MOOSE HSolve.  TEST INFRASTRUCTURE.
 *
 * The oracle for the GB300 HSolve: plain C, one thread, the reference's own
 * operation order (see hsolve_oracle.h for the list of reference functions
 * restated and their file:line).  Compile with -O2 -ffp-contract=off so that
 * every a*b+c is two IEEE roundings, as in the reference build.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU legs use this file.
 */
#include "hsolve_oracle.h"

#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ */
/* small growable arrays */
typedef struct { double* v; size_t n, cap; } dvec;
typedef struct { int64_t* v; size_t n, cap; } ivec;

static void dpush(dvec* a, double x) {
    if (a->n == a->cap) { a->cap = a->cap ? 2 * a->cap : 16; a->v = (double*)realloc(a->v, a->cap * sizeof(double)); }
    a->v[a->n++] = x;
}
static void ipush(ivec* a, int64_t x) {
    if (a->n == a->cap) { a->cap = a->cap ? 2 * a->cap : 16; a->v = (int64_t*)realloc(a->v, a->cap * sizeof(int64_t)); }
    a->v[a->n++] = x;
}
static void* xcalloc(size_t n, size_t s) { return calloc(n ? n : 1, s); }

/* ------------------------------------------------------------------ */
typedef struct { double* table; double min, max, dx; uint32_t nPts, nColumns; } LookupTable;
typedef struct { int64_t row; double fraction; } LookupRow;   /* row = offset into table */

typedef struct {
    double Gbar, Xpower, Ypower, Zpower, modulation;
    int instant;
} ChannelStruct;

typedef struct { double c, CaBasal, factor1, factor2, ceiling, floor_; } CaConcStruct;

typedef struct { uint32_t index, rank; } Junction;

/* External calcium objects on tick 1 (DifShell, DifBuffer, MMPump) and their
   messages, CSR by (source object, message kind) in description order. */
#define DIF_NK 6            /* object-sourced message kinds HS_DMSG_OUTER .. HS_DMSG_PUMP */
typedef struct {
    uint32_t n;
    double *C, *prevC, *dC, *Cm;                   /* DifShell C_, prevC_, dCbyDt_, Cmultiplier_ */
    double *bFree, *bBound, *prevFree, *Af, *Bf, *act;   /* DifBuffer */
    double *vol, *outerA, *innerA;                 /* geometry (calculateVolumeArea at reinit) */
    uint32_t *off, *dst;                           /* n*DIF_NK+1 */
    uint32_t *ikOff, *ikDst;                       /* by model HHChannel */
} DifObjs;

struct OrcCell {
    const HsCellDesc* d;        /* NULL for passive-only cells */
    double dt;                  /* HSolve dt_ */
    uint32_t nCompt;
    int caAdvance;
    int f32GateIncrements;      /* conditioning probe, see orc_set_f32_gate_increments */

    /* Hines order */
    uint32_t* compartmentId;    /* hines -> model */
    uint32_t* hinesOf;          /* model -> hines */
    double* V;
    double* CmByDt;
    double* EmByRm;
    /* inject_: map in the reference; dense here with a presence flag */
    uint8_t* injPresent;
    double* injectVarying;
    double* injectBasal;
    /* tree_ */
    uint32_t* childOff;         /* CSR, nCompt+1 */
    uint32_t* childIdx;
    double *Ra, *Rm, *Cm, *Em, *initVm;

    /* HinesMatrix; one memory block so that operand "pointers" are offsets:
       [0,4N) HS_, [4N,4N+H) HJ_, [4N+H, 5N+H) VMid_ */
    double* mem;
    size_t H;
    double* HJCopy;
    double* Ga;
    Junction* junction; size_t nJunction;
    /* coupled_ groups (sorted) */
    uint32_t* groupOff; uint32_t* groupIdx; size_t nGroup;
    int64_t* groupNumber;       /* per compt: group of a non-last member, or -1 */
    int64_t* operandBase;       /* per compt: offset of its HJ block (in mem), or -1 */
    ivec operand, backOperand;  /* offsets into mem */
    int stage;

    /* HSolveActive */
    uint32_t nChan;
    ChannelStruct* channel;
    double* Gk; double* Ek;     /* current_ */
    uint32_t* chanModel;        /* solver channel -> model channel */
    int64_t* chanSolverOf;      /* model channel -> solver channel */
    int* channelCount;
    uint32_t* currentBoundary;  /* cumulative channel counts per compartment */
    uint32_t* chan2compt;
    uint32_t* chan2state;
    dvec state;
    int* gCaDepend; size_t nGateIds; int64_t* gateId;
    uint32_t nPool;
    CaConcStruct* caConc;
    double* ca;
    double* caActivation;
    int64_t* caTarget;          /* per channel: index into caActivation or -1 */
    uint32_t* caCount;
    int64_t* caDependIndex;
    uint32_t* column;           /* per gate in gateId_ order */
    LookupRow* caRowCompt; uint32_t caRowComptSize;
    int64_t* caRow;             /* per Z gate: index into caRowCompt or -1 */
    double* externalCurrent;    /* 2N */
    double* prevExtCurr;
    double* externalCalcium;    /* per channel */
    uint32_t* poolModel;        /* solver pool -> model pool */
    int64_t* poolSolverOf;      /* model pool -> solver pool */
    LookupTable vTable, caTable;
    double vMin, vMax, caMin, caMax; int vDiv, caDiv;

    /* tick-4 external objects */
    double* c2dX; double* c2dVm; double* c2dConc1; double* c2dConc2; double* c2dGk;
    double* c2dMod; double* synMod;     /* modulation fields (ChanCommon), writable */
    double* synX; double* synY; double* synAct; double* synGk;
    double* synXc1; double* synXc2; double* synYc1; double* synYc2; double* synNorm;
    double* synDt;
    /* events per synchan, sorted by (time, input order) */
    uint32_t* evOff; double* evTime; double* evW; uint32_t* evPtr;
    /* events queued at run time (SimpleSynHandler::addSpike after reinit):
       per synchan a dvec pair sorted by (time, push order), consumed from
       rtHead; tick 1 pops the two queues in time order, description first
       on equal times */
    dvec* rtTime; dvec* rtW; uint32_t* rtHead;
    /* spikegens */
    double* sgLast; int* sgFired; uint32_t* sgComptHines; uint32_t nSg;
    ivec spikeGen; dvec spikeTime;
    /* stimulus */
    uint32_t stimPtr;
    /* tick-1 external calcium */
    DifObjs dif;

    double clockDt;
    uint64_t nSteps;
};

/* ------------------------------------------------------------------ */
/* LookupTable (hsolve/RateLookup.cpp:15-103) */
static void lt_init(LookupTable* t, double min, double max, uint32_t nDivs, uint32_t nSpecies) {
    t->min = min; t->max = max;
    t->nPts = nDivs + 1 + 1;
    t->dx = (max - min) / nDivs;
    t->nColumns = 2 * nSpecies;
    t->table = (double*)xcalloc((size_t)t->nPts * t->nColumns, sizeof(double));
}
static void lt_addColumns(LookupTable* t, int species, const double* C1, const double* C2, size_t n) {
    double* it = t->table + 2 * species;
    for (uint32_t igrid = 0; igrid < t->nPts - 1; ++igrid) {
        it[0] = C1[igrid]; it[1] = C2[igrid];
        it += t->nColumns;
    }
    it[0] = C1[n - 1]; it[1] = C2[n - 1];
}
static void lt_row(const LookupTable* t, double x, LookupRow* row) {
    if (x < t->min) x = t->min;
    else if (x > t->max) x = t->max;
    double div = (x - t->min) / t->dx;
    unsigned int integer = (unsigned int)(div);
    row->fraction = div - integer;
    row->row = (int64_t)integer * t->nColumns;
}
static void lt_lookup(const LookupTable* t, uint32_t column, const LookupRow* row, double* C1, double* C2) {
    const double* ap = t->table + row->row + column;
    const double* bp = ap + t->nColumns;
    double a = *ap, b = *bp;
    *C1 = a + (b - a) * row->fraction;
    a = *(ap + 1); b = *(bp + 1);
    *C2 = a + (b - a) * row->fraction;
}

/* HHGate::lookupBoth with interpolation (biophysics/HHGate.cpp:258-283) */
static void gate_lookupBoth(const HsGateTable* g, double v, double* A, double* B) {
    double invDx = (double)g->divs / (g->max - g->min);
    if (v <= g->min) { *A = g->A[0]; *B = g->B[0]; }
    else if (v >= g->max) { *A = g->A[g->divs]; *B = g->B[g->divs]; }
    else {
        unsigned int index = (unsigned int)((v - g->min) * invDx);
        double frac = (v - g->min - index / invDx) * invDx;
        *A = g->A[index] * (1 - frac) + g->A[index + 1] * frac;
        *B = g->B[index] * (1 - frac) + g->B[index + 1] * frac;
    }
}

/* ------------------------------------------------------------------ */
/* powers (hsolve/HSolveStruct.cpp:15-65) */
static double takePower(double x, double p) {
    if (p == 1.0) return x;
    if (p == 2.0) return x * x;
    if (p == 3.0) return x * x * x;
    if (p == 4.0) { double y = x * x; return y * y; }
    if (x > 0.0) return exp(p * log(x));
    return 0.0;
}

/* CaConcStruct (hsolve/HSolveStruct.cpp:108-155) */
static void ca_setTauB(CaConcStruct* s, double tau, double B, double dt) {
    s->factor1 = 4.0 / (2.0 + dt / tau) - 1.0;
    s->factor2 = 2.0 * B * dt / (2.0 + dt / tau);
}
static double ca_process(CaConcStruct* s, double activation) {
    s->c = s->factor1 * s->c + s->factor2 * activation;
    double ca = s->CaBasal + s->c;
    if (s->ceiling > 0 && ca > s->ceiling) { ca = s->ceiling; s->c = ca - s->CaBasal; }
    if (ca < s->floor_) { ca = s->floor_; s->c = ca - s->CaBasal; }
    return ca;
}

/* ------------------------------------------------------------------ */
/* Adjacency (HSolveUtils::adjacent, hsolve/HSolveUtils.cpp:36-45): axial
 * targets (axial children), raxial (the parent of an axial link), distalOut
 * (distal/sphere children), proximalOut (the parent of a SymCompartment
 * link), cylinderOut (cylinder children).  Children are kept in
 * HSolveUtils::children order (hsolve/HSolveUtils.cpp:47-53): by link kind,
 * increasing child index within a kind; e0/e1 end the axial and distal runs. */
typedef struct { uint32_t* off; uint32_t* idx; uint32_t* grp; } Adj;

static int link_of(const HsCellDesc* d, uint32_t i) { return d->link ? d->link[i] : HS_LINK_AXIAL; }

static Adj build_children(const HsCellDesc* d) {
    Adj a;
    uint32_t n = d->n_compt;
    a.off = (uint32_t*)xcalloc(n + 1, sizeof(uint32_t));
    for (uint32_t i = 0; i < n; i++) if (d->parent[i] >= 0) a.off[d->parent[i] + 1]++;
    for (uint32_t i = 0; i < n; i++) a.off[i + 1] += a.off[i];
    a.idx = (uint32_t*)xcalloc(a.off[n] + 1, sizeof(uint32_t));
    a.grp = (uint32_t*)xcalloc(2 * (size_t)n + 1, sizeof(uint32_t));
    uint32_t* fill = (uint32_t*)xcalloc(n + 1, sizeof(uint32_t));
    for (int kind = HS_LINK_AXIAL; kind <= HS_LINK_CYLINDER; kind++) {
        for (uint32_t i = 0; i < n; i++) if (d->parent[i] >= 0 && link_of(d, i) == kind) {
            uint32_t p = (uint32_t)d->parent[i];
            a.idx[a.off[p] + fill[p]++] = i;
        }
        if (kind < HS_LINK_CYLINDER)
            for (uint32_t p = 0; p < n; p++) a.grp[2 * p + kind] = a.off[p] + fill[p];
    }
    free(fill);
    return a;
}

static void adjacent(const HsCellDesc* d, const Adj* ch, uint32_t c, int64_t exclude, ivec* ret) {
    int has_parent = d->parent[c] >= 0 && (int64_t)d->parent[c] != exclude;
    int axial_up = link_of(d, c) == HS_LINK_AXIAL;
    uint32_t e0 = ch->grp[2 * c], e1 = ch->grp[2 * c + 1], end = ch->off[c + 1];
    for (uint32_t k = ch->off[c]; k < end; k++) {
        if (k == e0 && has_parent && axial_up) ipush(ret, d->parent[c]);
        if (k == e1 && has_parent && !axial_up) ipush(ret, d->parent[c]);
        if ((int64_t)ch->idx[k] != exclude) ipush(ret, ch->idx[k]);
    }
    if (has_parent && ((axial_up && e0 == end) || (!axial_up && e1 == end))) ipush(ret, d->parent[c]);
}

/* HSolvePassive::walkTree (hsolve/HSolvePassive.cpp:45-98) */
static int walkTree(OrcCell* c, const Adj* ch, uint32_t seed) {
    const HsCellDesc* d = c->d;
    ivec adj = {0};
    adjacent(d, ch, seed, -1, &adj);
    if (adj.n > 1) {
        uint32_t guard = 0;
        while (adj.n) {
            if (++guard > d->n_compt) { free(adj.v); return -1; }   /* a cycle */
            int64_t previous = seed;
            seed = (uint32_t)adj.v[0];
            adj.n = 0;
            adjacent(d, ch, seed, previous, &adj);
        }
    }
    free(adj.v);
    /* depth-first search with a stack of sibling stacks */
    size_t cap = 16, depth = 1;
    ivec* cstack = (ivec*)xcalloc(cap, sizeof(ivec));
    ipush(&cstack[0], seed);
    int64_t above = -1;
    uint32_t count = 0;
    uint32_t* order = (uint32_t*)xcalloc(d->n_compt, sizeof(uint32_t));
    while (depth) {
        ivec* top = &cstack[depth - 1];
        if (top->n == 0) {
            depth--;
            if (depth) cstack[depth - 1].n--;
        } else {
            if (depth > 1) above = cstack[depth - 2].v[cstack[depth - 2].n - 1];
            uint32_t current = (uint32_t)top->v[top->n - 1];
            if (count >= d->n_compt) { free(order); return -1; }   /* not a tree */
            order[count++] = current;
            if (depth == cap) {
                cstack = (ivec*)realloc(cstack, 2 * cap * sizeof(ivec));
                memset(cstack + cap, 0, cap * sizeof(ivec));
                cap *= 2;
            }
            cstack[depth].n = 0;
            adjacent(d, ch, current, above, &cstack[depth]);
            depth++;
        }
    }
    for (size_t i = 0; i < cap; i++) free(cstack[i].v);
    free(cstack);
    c->nCompt = count;
    c->compartmentId = (uint32_t*)xcalloc(count, sizeof(uint32_t));
    for (uint32_t i = 0; i < count; i++) c->compartmentId[i] = order[count - 1 - i];
    free(order);
    return 0;
}

/* ------------------------------------------------------------------ */
/* HinesMatrix (hsolve/HinesMatrix.cpp:25-365) */
static int cmp_u32(const void* a, const void* b) {
    uint32_t x = *(const uint32_t*)a, y = *(const uint32_t*)b;
    return x < y ? -1 : x > y;
}
typedef struct { uint32_t first; uint32_t seq; uint32_t* m; uint32_t n; } GroupTmp;
static int cmp_group(const void* a, const void* b) {
    const GroupTmp* x = (const GroupTmp*)a; const GroupTmp* y = (const GroupTmp*)b;
    if (x->first != y->first) return x->first < y->first ? -1 : 1;
    return x->seq < y->seq ? -1 : x->seq > y->seq;
}
static int cmp_junction(const void* a, const void* b) {
    const Junction* x = (const Junction*)a; const Junction* y = (const Junction*)b;
    return x->index < y->index ? -1 : x->index > y->index;
}

#define HS(i) (c->mem[(i)])

static void hines_setup(OrcCell* c) {
    uint32_t n = c->nCompt;
    c->Ga = (double*)xcalloc(n, sizeof(double));
    for (uint32_t i = 0; i < n; i++) c->Ga[i] = 2.0 / c->Ra[i];

    /* makeJunctions */
    GroupTmp* g = (GroupTmp*)xcalloc(n, sizeof(GroupTmp));
    size_t ng = 0;
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t nc = c->childOff[i + 1] - c->childOff[i];
        const uint32_t* ch = c->childIdx + c->childOff[i];
        if (nc == 0) continue;
        if (nc == 1) {
            int diff = (int)ch[0] - (int)i;
            if (diff == 1 || diff == -1) continue;
        }
        g[ng].m = (uint32_t*)xcalloc(nc + 1, sizeof(uint32_t));
        memcpy(g[ng].m, ch, nc * sizeof(uint32_t));
        g[ng].m[nc] = i;
        g[ng].n = nc + 1;
        g[ng].seq = (uint32_t)ng;
        ng++;
    }
    for (size_t k = 0; k < ng; k++) { qsort(g[k].m, g[k].n, sizeof(uint32_t), cmp_u32); g[k].first = g[k].m[0]; }
    /* std::sort with groupCompare: groups have distinct first elements */
    qsort(g, ng, sizeof(GroupTmp), cmp_group);
    c->nGroup = ng;
    c->groupOff = (uint32_t*)xcalloc(ng + 1, sizeof(uint32_t));
    for (size_t k = 0; k < ng; k++) c->groupOff[k + 1] = c->groupOff[k] + g[k].n;
    c->groupIdx = (uint32_t*)xcalloc(c->groupOff[ng], sizeof(uint32_t));
    for (size_t k = 0; k < ng; k++) { memcpy(c->groupIdx + c->groupOff[k], g[k].m, g[k].n * sizeof(uint32_t)); free(g[k].m); }
    free(g);

    c->groupNumber = (int64_t*)xcalloc(n, sizeof(int64_t));
    for (uint32_t i = 0; i < n; i++) c->groupNumber[i] = -1;
    c->junction = (Junction*)xcalloc(c->groupOff[ng], sizeof(Junction));
    c->nJunction = 0;
    for (size_t k = 0; k < ng; k++) {
        uint32_t sz = c->groupOff[k + 1] - c->groupOff[k];
        for (uint32_t m = 0; m < sz - 1; ++m) {
            uint32_t index = c->groupIdx[c->groupOff[k] + m];
            c->junction[c->nJunction].index = index;
            c->junction[c->nJunction].rank = sz - m - 1;
            c->nJunction++;
            c->groupNumber[index] = (int64_t)k;
        }
    }
    qsort(c->junction, c->nJunction, sizeof(Junction), cmp_junction);

    /* makeMatrix */
    size_t H = 0;
    for (size_t k = 0; k < ng; k++) {
        size_t rank = c->groupOff[k + 1] - c->groupOff[k] - 1;
        H += rank * (rank + 1);
    }
    c->H = H;
    c->mem = (double*)xcalloc(4 * (size_t)n + H + n, sizeof(double));
    for (uint32_t i = 0; i < n; ++i)
        HS(4 * i + 2) = c->Cm[i] / (c->dt / 2.0) + 1.0 / c->Rm[i];
    size_t jn = 0;
    for (uint32_t i = 0; i + 1 < n; ++i) {
        if (c->nJunction && jn < c->nJunction && i == c->junction[jn].index) { ++jn; continue; }
        double gi = c->Ga[i], gj = c->Ga[i + 1];
        double gij = gi * gj / (gi + gj);
        HS(4 * i + 1) = -gij;
        HS(4 * i + 2) += gij;
        HS(4 * i + 6) += gij;
    }
    for (size_t k = 0; k < ng; k++) {
        double gsum = 0.0;
        for (uint32_t q = c->groupOff[k]; q < c->groupOff[k + 1]; q++) gsum += c->Ga[c->groupIdx[q]];
        for (uint32_t q = c->groupOff[k]; q < c->groupOff[k + 1]; q++) {
            double gi = c->Ga[c->groupIdx[q]];
            HS(4 * c->groupIdx[q] + 2) += gi * (1.0 - gi / gsum);
        }
    }
    c->operandBase = (int64_t*)xcalloc(n, sizeof(int64_t));
    for (uint32_t i = 0; i < n; i++) c->operandBase[i] = -1;
    size_t hj = 0;
    const size_t hjBase = 4 * (size_t)n;
    for (size_t k = 0; k < ng; k++) {
        double gsum = 0.0;
        for (uint32_t q = c->groupOff[k]; q < c->groupOff[k + 1]; q++) gsum += c->Ga[c->groupIdx[q]];
        for (uint32_t q = c->groupOff[k]; q + 1 < c->groupOff[k + 1]; q++) {
            size_t base = hj;
            for (uint32_t r = q + 1; r < c->groupOff[k + 1]; r++) {
                double gij = c->Ga[c->groupIdx[q]] * c->Ga[c->groupIdx[r]] / gsum;
                HS(hjBase + hj++) = -gij;
                HS(hjBase + hj++) = -gij;
            }
            c->operandBase[c->groupIdx[q]] = (int64_t)(hjBase + base);
        }
    }
    for (uint32_t i = 0; i < n; ++i) HS(4 * i) = HS(4 * i + 2);
    c->HJCopy = (double*)xcalloc(H, sizeof(double));
    memcpy(c->HJCopy, c->mem + hjBase, H * sizeof(double));

    /* makeOperands */
    const int64_t vmid = (int64_t)(4 * (size_t)n + H);
    for (size_t jk = 0; jk < c->nJunction; jk++) {
        uint32_t index = c->junction[jk].index, rank = c->junction[jk].rank;
        int64_t base = c->operandBase[index];
        int64_t gnum = c->groupNumber[index];
        const uint32_t* group = c->groupIdx + c->groupOff[gnum];
        uint32_t gsize = c->groupOff[gnum + 1] - c->groupOff[gnum];
        if (rank == 1) {
            ipush(&c->operand, base);
            uint32_t far = group[gsize - 1];
            ipush(&c->operand, 4 * (int64_t)far);
            ipush(&c->operand, vmid + far);
        } else if (rank == 2) {
            ipush(&c->operand, base);
            uint32_t far = group[gsize - 2];
            ipush(&c->operand, 4 * (int64_t)far);
            ipush(&c->operand, vmid + far);
            far = group[gsize - 1];
            ipush(&c->operand, 4 * (int64_t)far);
            ipush(&c->operand, vmid + far);
        } else {
            int start = (int)gsize - (int)rank;
            for (uint32_t j = 0; j < rank; ++j) {
                uint32_t far = group[start + j];
                ipush(&c->operand, 4 * (int64_t)far);
                ipush(&c->operand, base + 2 * j);
                ipush(&c->operand, base + 2 * j + 1);
                ipush(&c->operand, 4 * (int64_t)far + 3);
                ipush(&c->operand, 4 * (int64_t)index + 3);
                ipush(&c->operand, base + 2 * j + 1);
            }
            int64_t left = base + 1, target = base + 2 * rank, above;
            for (uint32_t i = 1; i < rank; ++i) {
                above = base + 2 * i;
                for (uint32_t j = 0; j < rank - i; ++j) {
                    ipush(&c->operand, target); ipush(&c->operand, above); ipush(&c->operand, left);
                    above += 2; target += 2;
                }
                left += 2;
            }
            target = base + 2 * rank + 1;
            above = base;
            for (uint32_t i = 1; i < rank; ++i) {
                left = base + 2 * i + 1;
                for (uint32_t j = 0; j < rank - i; ++j) {
                    ipush(&c->operand, target); ipush(&c->operand, above); ipush(&c->operand, left);
                    if (i == rank - 1 && j == rank - i - 1) continue;
                    target += 2; left += 2;
                }
                above += 2;
            }
        }
    }
    for (size_t jk = 0; jk < c->nJunction; jk++) {
        if (c->junction[jk].rank < 3) continue;
        uint32_t index = c->junction[jk].index, rank = c->junction[jk].rank;
        int64_t base = c->operandBase[index];
        int64_t gnum = c->groupNumber[index];
        const uint32_t* group = c->groupIdx + c->groupOff[gnum];
        uint32_t gsize = c->groupOff[gnum + 1] - c->groupOff[gnum];
        uint32_t start = gsize - rank;
        for (uint32_t j = 0; j < rank; ++j) {
            uint32_t far = group[start + j];
            ipush(&c->backOperand, base + 2 * j);
            ipush(&c->backOperand, vmid + far);
        }
    }
    c->stage = -1;
}

/* HSolvePassive::forwardEliminate (hsolve/HSolvePassive.cpp:246-323) */
void orc_forward(OrcCell* c) {
    uint32_t ic = 0;
    size_t ihs = 0;
    size_t iop = 0;
    double* m = c->mem;
    const int64_t* op = c->operand.v;
    for (size_t jk = 0; jk < c->nJunction; jk++) {
        uint32_t index = c->junction[jk].index, rank = c->junction[jk].rank;
        while (ic < index) {
            m[ihs + 4] -= m[ihs + 1] / m[ihs] * m[ihs + 1];
            m[ihs + 7] -= m[ihs + 1] / m[ihs] * m[ihs + 3];
            ++ic, ihs += 4;
        }
        double pivot = m[ihs];
        if (rank == 1) {
            int64_t j = op[iop], s = op[iop + 1];
            double division = m[j + 1] / pivot;
            m[s] -= division * m[j];
            m[s + 3] -= division * m[ihs + 3];
            iop += 3;
        } else if (rank == 2) {
            int64_t j = op[iop], s;
            s = op[iop + 1];
            double division = m[j + 1] / pivot;
            m[s] -= division * m[j];
            m[j + 4] -= division * m[j + 2];
            m[s + 3] -= division * m[ihs + 3];
            s = op[iop + 3];
            division = m[j + 3] / pivot;
            m[j + 5] -= division * m[j];
            m[s] -= division * m[j + 2];
            m[s + 3] -= division * m[ihs + 3];
            iop += 5;
        } else {
            size_t end = iop + 3 * (size_t)rank * (rank + 1);
            for (; iop < end; iop += 3)
                m[op[iop]] -= m[op[iop + 2]] / pivot * m[op[iop + 1]];
        }
        ++ic, ihs += 4;
    }
    while (ic + 1 < c->nCompt) {
        m[ihs + 4] -= m[ihs + 1] / m[ihs] * m[ihs + 1];
        m[ihs + 7] -= m[ihs + 1] / m[ihs] * m[ihs + 3];
        ++ic, ihs += 4;
    }
    c->stage = 1;
}

/* HSolvePassive::backwardSubstitute (hsolve/HSolvePassive.cpp:325-401);
 * the reverse iterators become explicit descending indices. */
void orc_backward(OrcCell* c) {
    uint32_t n = c->nCompt;
    double* m = c->mem;
    double* VMid = c->mem + 4 * (size_t)n + c->H;
    double* V = c->V;
    const int64_t* op = c->operand.v;
    const int64_t* bop = c->backOperand.v;
    int64_t iop = (int64_t)c->operand.n - 1;      /* *(iop+k) == op[iop-k] */
    int64_t ibop = (int64_t)c->backOperand.n - 1;
    int ic = (int)n - 1;
    VMid[ic] = m[4 * ic + 3] / m[4 * ic];
    V[ic] = 2 * VMid[ic] - V[ic];
    --ic;
    for (int64_t jk = (int64_t)c->nJunction - 1; jk >= 0; jk--) {
        int index = (int)c->junction[jk].index, rank = (int)c->junction[jk].rank;
        while (ic > index) {
            VMid[ic] = (m[4 * ic + 3] - m[4 * ic + 1] * VMid[ic + 1]) / m[4 * ic];
            V[ic] = 2 * VMid[ic] - V[ic];
            --ic;
        }
        if (rank == 1) {
            VMid[ic] = (m[4 * ic + 3] - m[op[iop]] * m[op[iop - 2]]) / m[4 * ic];
            iop -= 3;
        } else if (rank == 2) {
            int64_t v0 = op[iop], v1 = op[iop - 2], j = op[iop - 4];
            VMid[ic] = (m[4 * ic + 3] - m[v0] * m[j + 2] - m[v1] * m[j]) / m[4 * ic];
            iop -= 5;
        } else {
            double v = m[4 * ic + 3];
            for (int i = 0; i < rank; ++i) {
                v -= m[bop[ibop]] * m[bop[ibop - 1]];
                ibop -= 2;
            }
            v /= m[4 * ic];
            VMid[ic] = v;
            iop -= 3 * (int64_t)rank * (rank + 1);
        }
        V[ic] = 2 * VMid[ic] - V[ic];
        --ic;
    }
    while (ic >= 0) {
        VMid[ic] = (m[4 * ic + 3] - m[4 * ic + 1] * VMid[ic + 1]) / m[4 * ic];
        V[ic] = 2 * VMid[ic] - V[ic];
        --ic;
    }
    c->stage = 2;
}

/* HSolvePassive::updateMatrix (hsolve/HSolvePassive.cpp:211-244) */
void orc_passive_update(OrcCell* c) {
    uint32_t n = c->nCompt;
    if (c->H) memcpy(c->mem + 4 * (size_t)n, c->HJCopy, c->H * sizeof(double));
    for (uint32_t i = 0; i < n; i++) {
        HS(4 * i) = HS(4 * i + 2);
        HS(4 * i + 3) = c->V[i] * c->CmByDt[i] + c->EmByRm[i];
    }
    for (uint32_t i = 0; i < n; i++) if (c->injPresent[i]) {
        HS(4 * i + 3) += c->injectVarying[i] + c->injectBasal[i];
        c->injectVarying[i] = 0.0;
    }
    c->stage = 0;
}

/* HinesMatrix::getA (hsolve/HinesMatrix.cpp:375-434) */
double orc_getA(const OrcCell* c, uint32_t row, uint32_t col) {
    if ((c->stage == 1 || c->stage == 2) && row > col) return 0.0;
    if (row >= c->nCompt || col >= c->nCompt) return 0.0;
    if (row == col) return c->mem[4 * row];
    uint32_t smaller = row < col ? row : col, bigger = row > col ? row : col;
    if (c->groupNumber[smaller] < 0) {
        if (bigger - smaller == 1) return c->mem[4 * smaller + 1];
        return 0.0;
    }
    int64_t gnum = c->groupNumber[smaller];
    const uint32_t* group = c->groupIdx + c->groupOff[gnum];
    uint32_t size = c->groupOff[gnum + 1] - c->groupOff[gnum];
    int found = 0;
    uint32_t ps = 0, pb = 0;
    for (uint32_t q = 0; q < size; q++) {
        if (group[q] == bigger) { found = 1; pb = q; }
        if (group[q] == smaller) ps = q;
    }
    if (!found) return 0.0;
    size_t location = 0;
    for (int64_t i = 0; i < gnum; ++i) {
        size_t s = c->groupOff[i + 1] - c->groupOff[i];
        location += s * (s - 1);
    }
    uint32_t smallRank = size - ps - 1, bigRank = size - pb - 1;
    location += (size_t)size * (size - 1) - (size_t)smallRank * (smallRank + 1);
    location += 2 * (smallRank - bigRank - 1);
    const double* HJ = c->mem + 4 * (size_t)c->nCompt;
    return row == smaller ? HJ[location] : HJ[location + 1];
}
double orc_getB(const OrcCell* c, uint32_t row) { return c->mem[4 * row + 3]; }
double orc_getVMid(const OrcCell* c, uint32_t row) { return c->mem[4 * (size_t)c->nCompt + c->H + row]; }
double orc_getV(const OrcCell* c, uint32_t row) { return c->V[row]; }

OrcCell* orc_passive_create(uint32_t n, const uint32_t* child_off, const uint32_t* child_idx,
                            const double* Ra, const double* Rm, const double* Cm,
                            const double* Em, const double* V, double dt) {
    OrcCell* c = (OrcCell*)xcalloc(1, sizeof(OrcCell));
    c->dt = dt; c->nCompt = n;
    c->childOff = (uint32_t*)xcalloc(n + 1, sizeof(uint32_t));
    memcpy(c->childOff, child_off, (n + 1) * sizeof(uint32_t));
    c->childIdx = (uint32_t*)xcalloc(child_off[n], sizeof(uint32_t));
    memcpy(c->childIdx, child_idx, child_off[n] * sizeof(uint32_t));
    c->Ra = (double*)xcalloc(n, sizeof(double)); memcpy(c->Ra, Ra, n * sizeof(double));
    c->Rm = (double*)xcalloc(n, sizeof(double)); memcpy(c->Rm, Rm, n * sizeof(double));
    c->Cm = (double*)xcalloc(n, sizeof(double)); memcpy(c->Cm, Cm, n * sizeof(double));
    c->Em = (double*)xcalloc(n, sizeof(double)); memcpy(c->Em, Em, n * sizeof(double));
    c->V = (double*)xcalloc(n, sizeof(double)); memcpy(c->V, V, n * sizeof(double));
    c->CmByDt = (double*)xcalloc(n, sizeof(double));
    c->EmByRm = (double*)xcalloc(n, sizeof(double));
    c->injPresent = (uint8_t*)xcalloc(n, 1);
    c->injectVarying = (double*)xcalloc(n, sizeof(double));
    c->injectBasal = (double*)xcalloc(n, sizeof(double));
    for (uint32_t i = 0; i < n; i++) {
        c->CmByDt[i] = 2.0 * Cm[i] / dt;
        c->EmByRm[i] = Em[i] / Rm[i];
    }
    hines_setup(c);
    return c;
}

/* ------------------------------------------------------------------ */
/* HSolveActive::setup (hsolve/HSolveActiveSetup.cpp:17-41) */
static int cmp_i64(const void* a, const void* b) {
    int64_t x = *(const int64_t*)a, y = *(const int64_t*)b;
    return x < y ? -1 : x > y;
}

/* ------------------------------------------------------------------ */
/* External calcium on tick 1: DifShell (biophysics/DifShell.cpp), DifBuffer
   (biophysics/DifBuffer.cpp), MMPump (biophysics/MMPump.cpp).  Each object
   processes in tick order and its sends reach their targets at once, so a
   target processed later in the same tick sees this step's value. */
static const double DIF_F = 96485.3415;        /* DifShell::F */
static const double DIF_EPSILON = 1.0e-10;     /* DifShell::EPSILON, DifBuffer::EPSILON */
static const double DIF_PI = 3.14159265358979323846;   /* M_PI of the reference's <cmath> */
#define DP(k, i) (c->d->difpar[(size_t)(k) * HS_DIF_NPAR + (i)])

static const char* dif_setup(OrcCell* c) {
    const HsCellDesc* d = c->d;
    DifObjs* o = &c->dif;
    uint32_t n = d->n_dif;
    o->n = n;
    if (!n && !d->n_dmsg) return NULL;
    if (n && (!d->dif_kind || !d->difpar)) return "tick-1 objects without kinds or parameters";
    for (uint32_t k = 0; k < n; k++)
        if (d->dif_kind[k] < HS_DIF_SHELL || d->dif_kind[k] > HS_DIF_PUMP) return "unknown tick-1 object kind";
    double** arrs[] = {&o->C, &o->prevC, &o->dC, &o->Cm, &o->bFree, &o->bBound, &o->prevFree, &o->Af, &o->Bf,
                       &o->act, &o->vol, &o->outerA, &o->innerA};
    for (size_t a = 0; a < sizeof(arrs) / sizeof(arrs[0]); a++) *arrs[a] = (double*)xcalloc(n, sizeof(double));
    for (uint32_t k = 0; k < n; k++) if (d->dif_kind[k] == HS_DIF_BUFFER) o->act[k] = DP(k, 11);
    o->off = (uint32_t*)xcalloc((size_t)n * DIF_NK + 1, sizeof(uint32_t));
    o->ikOff = (uint32_t*)xcalloc((size_t)d->n_chan + 1, sizeof(uint32_t));
    for (uint32_t m = 0; m < d->n_dmsg; m++) {
        int kind = d->dmsg_kind[m];
        uint32_t s = d->dmsg_src[m], t = d->dmsg_dst[m];
        if (kind == HS_DMSG_IK) {
            if (s >= d->n_chan || c->chanSolverOf[s] < 0) return "IkOut from a channel the solver does not hold";
            if (t >= n || d->dif_kind[t] != HS_DIF_SHELL) return "IkOut to an object that is not a DifShell";
            o->ikOff[s + 1]++;
            continue;
        }
        if (kind < HS_DMSG_OUTER || kind > HS_DMSG_PUMP || s >= n) return "bad tick-1 message";
        int sk = d->dif_kind[s];
        int ok;
        switch (kind) {
        case HS_DMSG_OUTER: case HS_DMSG_INNER:
            ok = sk != HS_DIF_PUMP && t < n && d->dif_kind[t] != HS_DIF_PUMP; break;
        case HS_DMSG_CONC_CHAN:
            ok = sk == HS_DIF_SHELL && t < d->n_chan && c->chanSolverOf[t] >= 0; break;
        case HS_DMSG_CONC_BUF:
            ok = sk == HS_DIF_SHELL && t < n && d->dif_kind[t] == HS_DIF_BUFFER; break;
        case HS_DMSG_REACTION:
            ok = sk == HS_DIF_BUFFER && t < n && d->dif_kind[t] == HS_DIF_SHELL; break;
        default:  /* HS_DMSG_PUMP */
            ok = sk == HS_DIF_PUMP && t < n && d->dif_kind[t] == HS_DIF_SHELL; break;
        }
        if (!ok) return "tick-1 message between objects of the wrong kinds";
        o->off[(size_t)s * DIF_NK + kind + 1]++;
    }
    for (size_t i = 0; i < (size_t)n * DIF_NK; i++) o->off[i + 1] += o->off[i];
    for (uint32_t k = 0; k < d->n_chan; k++) o->ikOff[k + 1] += o->ikOff[k];
    o->dst = (uint32_t*)xcalloc(o->off[(size_t)n * DIF_NK] + 1, sizeof(uint32_t));
    o->ikDst = (uint32_t*)xcalloc(o->ikOff[d->n_chan] + 1, sizeof(uint32_t));
    uint32_t* fill = (uint32_t*)xcalloc((size_t)n * DIF_NK + d->n_chan + 1, sizeof(uint32_t));
    for (uint32_t m = 0; m < d->n_dmsg; m++) {
        uint32_t s = d->dmsg_src[m];
        if (d->dmsg_kind[m] == HS_DMSG_IK) {
            o->ikDst[o->ikOff[s] + fill[(size_t)n * DIF_NK + s]++] = d->dmsg_dst[m];
        } else {
            size_t slot = (size_t)s * DIF_NK + d->dmsg_kind[m];
            o->dst[o->off[slot] + fill[slot]++] = d->dmsg_dst[m];
        }
    }
    free(fill);
    return NULL;
}

/* DifShell::calculateVolumeArea and the same in DifBuffer::vReinit */
static void dif_geometry(OrcCell* c, uint32_t k) {
    DifObjs* o = &c->dif;
    int shape = (int)DP(k, 4);
    double length = DP(k, 5), diameter = DP(k, 6), thickness = DP(k, 7);
    double rOut = diameter / 2.;
    double rIn = rOut - thickness;
    if (rIn < 0) rIn = 0.;
    if (shape == 0) {
        if (length == 0.0) {
            o->vol[k] = 4. / 3. * DIF_PI * (rOut * rOut * rOut - rIn * rIn * rIn);
            o->outerA[k] = 4 * DIF_PI * rOut * rOut;
            o->innerA[k] = 4 * DIF_PI * rIn * rIn;
        } else {
            o->vol[k] = (DIF_PI * length) * (rOut * rOut - rIn * rIn);
            o->outerA[k] = 2 * DIF_PI * rOut * length;
            o->innerA[k] = 2 * DIF_PI * rIn * length;
        }
    } else if (shape == 1) {
        o->vol[k] = DIF_PI * diameter * diameter * thickness / 4.0;
        o->outerA[k] = DIF_PI * diameter * diameter / 4.0;
        o->innerA[k] = o->outerA[k];
    } else {    /* 3: user defined */
        o->vol[k] = DP(k, 8);
        o->outerA[k] = DP(k, 9);
        o->innerA[k] = DP(k, 10);
    }
}

/* DifShell::integrate, DifBuffer::integrate */
static double dif_integrate(double state, double dt, double A, double B) {
    if (B > DIF_EPSILON) {
        double x = exp(-B * dt);
        return state * x + (A / B) * (1 - x);
    }
    return state + A * dt;
}

/* inner/outerDifSourceOut of object s: fluxFromIn/Out of each target */
static void dif_send_flux(OrcCell* c, uint32_t s, int kind, double value, double thickness) {
    DifObjs* o = &c->dif;
    size_t slot = (size_t)s * DIF_NK + kind;
    for (uint32_t i = o->off[slot]; i < o->off[slot + 1]; i++) {
        uint32_t t = o->dst[i];
        double D = c->d->dif_kind[t] == HS_DIF_SHELL ? DP(t, 1) : DP(t, 3);
        double area = kind == HS_DMSG_OUTER ? o->outerA[t] : o->innerA[t];
        double tt = DP(t, 7);
        if (c->d->dif_kind[t] == HS_DIF_SHELL) {
            /* vFluxFromOut / vFluxFromIn */
            double diff = 2. * D / o->vol[t] * area / (thickness + tt);
            o->dC[t] += diff * value;
            o->Cm[t] += diff;
        } else {
            double dif = 2 * D / o->vol[t] * area / (tt + thickness);
            o->Af[t] += dif * value;
            o->Bf[t] += dif;
        }
    }
}

/* concentrationOut of shell s: HHChannel concen (HSolve::addConc) and
   DifBuffer concentration (vBuffer: activation) */
static void dif_send_conc(OrcCell* c, uint32_t s, double C) {
    DifObjs* o = &c->dif;
    size_t slot = (size_t)s * DIF_NK + HS_DMSG_CONC_CHAN;
    for (uint32_t i = o->off[slot]; i < o->off[slot + 1]; i++)
        c->externalCalcium[c->chanSolverOf[o->dst[i]]] = C;
    slot = (size_t)s * DIF_NK + HS_DMSG_CONC_BUF;
    for (uint32_t i = o->off[slot]; i < o->off[slot + 1]; i++) o->act[o->dst[i]] = C;
}

/* every object's reinit, tick order (DifShell::vReinit, DifBuffer::vReinit;
   MMPump::reinit does nothing) */
static void dif_reinit(OrcCell* c) {
    DifObjs* o = &c->dif;
    for (uint32_t k = 0; k < o->n; k++) {
        int kind = c->d->dif_kind[k];
        if (kind == HS_DIF_SHELL) {
            o->dC[k] = DP(k, 3);
            o->Cm[k] = 0;
            dif_geometry(c, k);
            o->C[k] = DP(k, 0);
            o->prevC[k] = DP(k, 0);
            dif_send_conc(c, k, o->C[k]);
            dif_send_flux(c, k, HS_DMSG_INNER, o->prevC[k], DP(k, 7));
            dif_send_flux(c, k, HS_DMSG_OUTER, o->prevC[k], DP(k, 7));
        } else if (kind == HS_DIF_BUFFER) {
            o->Af[k] = 0;
            o->Bf[k] = 0;
            dif_geometry(c, k);
            double bTot = DP(k, 0), kf = DP(k, 1), kb = DP(k, 2);
            o->bFree[k] = bTot / (1 + o->act[k] * kf / kb);
            o->prevFree[k] = o->bFree[k];
            o->bBound[k] = bTot - o->bFree[k];
            dif_send_flux(c, k, HS_DMSG_INNER, o->prevFree[k], DP(k, 7));
            dif_send_flux(c, k, HS_DMSG_OUTER, o->prevFree[k], DP(k, 7));
        }
    }
}

/* every object's process, tick order (DifShell::vProcess,
   DifBuffer::vProcess, MMPump::process) */
static void dif_process(OrcCell* c, double dt) {
    DifObjs* o = &c->dif;
    for (uint32_t k = 0; k < o->n; k++) {
        int kind = c->d->dif_kind[k];
        if (kind == HS_DIF_SHELL) {
            o->C[k] = dif_integrate(o->C[k], dt, o->dC[k], o->Cm[k]);
            o->dC[k] = DP(k, 3);
            o->Cm[k] = 0;
            o->prevC[k] = o->C[k];
            dif_send_flux(c, k, HS_DMSG_INNER, o->prevC[k], DP(k, 7));
            dif_send_flux(c, k, HS_DMSG_OUTER, o->prevC[k], DP(k, 7));
            dif_send_conc(c, k, o->C[k]);
        } else if (kind == HS_DIF_BUFFER) {
            double bTot = DP(k, 0), kf = DP(k, 1), kb = DP(k, 2);
            o->Af[k] += kb * o->bBound[k];
            o->Bf[k] += kf * o->act[k];
            o->bFree[k] = dif_integrate(o->bFree[k], dt, o->Af[k], o->Bf[k]);
            o->bBound[k] = bTot - o->bFree[k];
            o->prevFree[k] = o->bFree[k];
            dif_send_flux(c, k, HS_DMSG_INNER, o->prevFree[k], DP(k, 7));
            dif_send_flux(c, k, HS_DMSG_OUTER, o->prevFree[k], DP(k, 7));
            /* reactionOut -> DifShell::vBuffer */
            size_t slot = (size_t)k * DIF_NK + HS_DMSG_REACTION;
            for (uint32_t i = o->off[slot]; i < o->off[slot + 1]; i++) {
                uint32_t t = o->dst[i];
                o->dC[t] += kb * o->bBound[k];
                o->Cm[t] += kf * o->bFree[k];
            }
            o->Af[k] = 0;
            o->Bf[k] = 0;
        } else {
            /* PumpOut -> DifShell::vMMPump */
            double vMax = DP(k, 0), Kd = DP(k, 1);
            size_t slot = (size_t)k * DIF_NK + HS_DMSG_PUMP;
            for (uint32_t i = o->off[slot]; i < o->off[slot + 1]; i++) {
                uint32_t t = o->dst[i];
                o->Cm[t] += (vMax / o->vol[t]) / (o->C[t] + Kd);
            }
        }
    }
}

/* HSolveActive::sendValues, IkOut (hsolve/HSolveActive.cpp:367-376):
   (Ek - Vm) Gk of each channel, channel order, to DifShell::vInflux */
static void dif_send_ik(OrcCell* c) {
    DifObjs* o = &c->dif;
    if (!o->ikOff) return;
    for (uint32_t q = 0; q < c->nChan; q++) {
        uint32_t k = c->chanModel[q];
        if (o->ikOff[k] == o->ikOff[k + 1]) continue;
        double I = (c->Ek[q] - c->V[c->chan2compt[q]]) * c->Gk[q];
        for (uint32_t i = o->ikOff[k]; i < o->ikOff[k + 1]; i++) {
            uint32_t t = o->ikDst[i];
            o->dC[t] += I / (DIF_F * DP(t, 2) * o->vol[t]);
        }
    }
}

OrcCell* orc_create(const HsCellDesc* d, uint32_t seed, double dt, char* err, uint32_t errlen) {
#define FAIL(msg) do { if (err && errlen) snprintf(err, errlen, "%s", msg); orc_destroy(c); return NULL; } while (0)
    OrcCell* c = (OrcCell*)xcalloc(1, sizeof(OrcCell));
    c->d = d; c->dt = dt; c->caAdvance = 1;
    if (!d || d->n_compt == 0) FAIL("empty cell");
    if (seed >= d->n_compt) FAIL("seed out of range");
    if (!(dt > 0)) FAIL("dt must be positive");
    for (uint32_t i = 0; i < d->n_compt; i++) {
        if (d->parent[i] >= (int32_t)d->n_compt || d->parent[i] == (int32_t)i) FAIL("bad parent index");
        if (d->link && (d->link[i] < HS_LINK_AXIAL || d->link[i] > HS_LINK_CYLINDER)) FAIL("bad link kind");
    }
    Adj ch = build_children(d);
    if (walkTree(c, &ch, seed) != 0) { free(ch.off); free(ch.idx); free(ch.grp); FAIL("compartment graph is not a tree"); }
    uint32_t n = c->nCompt;
    c->hinesOf = (uint32_t*)xcalloc(d->n_compt, sizeof(uint32_t));
    for (uint32_t i = 0; i < d->n_compt; i++) c->hinesOf[i] = UINT32_MAX;
    for (uint32_t i = 0; i < n; i++) c->hinesOf[c->compartmentId[i]] = i;

    /* initialize (hsolve/HSolvePassive.cpp:100-165) */
    c->V = (double*)xcalloc(n, sizeof(double));
    c->CmByDt = (double*)xcalloc(n, sizeof(double));
    c->EmByRm = (double*)xcalloc(n, sizeof(double));
    c->injPresent = (uint8_t*)xcalloc(n, 1);
    c->injectVarying = (double*)xcalloc(n, sizeof(double));
    c->injectBasal = (double*)xcalloc(n, sizeof(double));
    for (uint32_t ic = 0; ic < n; ++ic) {
        uint32_t m = c->compartmentId[ic];
        c->V[ic] = d->Vm[m];
        double EmGmThev = d->Em[m] / d->Rm[m];
        for (uint32_t l = 0; l < d->n_leak; l++) if (d->leak_compt[l] == m)
            EmGmThev += d->leak_Ek[l] * d->leak_Gk[l];
        c->CmByDt[ic] = 2.0 * d->Cm[m] / dt;
        c->EmByRm[ic] = EmGmThev;
        if (d->inject[m] != 0.0) { c->injPresent[ic] = 1; c->injectVarying[ic] = 0.0; c->injectBasal[ic] = d->inject[m]; }
    }
    /* storeTree (hsolve/HSolvePassive.cpp:167-205) */
    c->childOff = (uint32_t*)xcalloc(n + 1, sizeof(uint32_t));
    for (uint32_t ic = 0; ic < n; ic++) {
        uint32_t m = c->compartmentId[ic];
        c->childOff[ic + 1] = c->childOff[ic] + (ch.off[m + 1] - ch.off[m]);
    }
    c->childIdx = (uint32_t*)xcalloc(c->childOff[n], sizeof(uint32_t));
    c->Ra = (double*)xcalloc(n, sizeof(double)); c->Rm = (double*)xcalloc(n, sizeof(double));
    c->Cm = (double*)xcalloc(n, sizeof(double)); c->Em = (double*)xcalloc(n, sizeof(double));
    c->initVm = (double*)xcalloc(n, sizeof(double));
    for (uint32_t ic = 0; ic < n; ic++) {
        uint32_t m = c->compartmentId[ic];
        for (uint32_t k = ch.off[m]; k < ch.off[m + 1]; k++)
            c->childIdx[c->childOff[ic] + (k - ch.off[m])] = c->hinesOf[ch.idx[k]];
        c->Ra[ic] = d->Ra[m]; c->Rm[ic] = d->Rm[m]; c->Cm[ic] = d->Cm[m];
        c->Em[ic] = d->Em[m]; c->initVm[ic] = d->initVm[m];
    }
    free(ch.off); free(ch.idx); free(ch.grp);
    hines_setup(c);

    /* readHHChannels (hsolve/HSolveActiveSetup.cpp:162-235) */
    c->channelCount = (int*)xcalloc(n, sizeof(int));
    c->chanSolverOf = (int64_t*)xcalloc(d->n_chan, sizeof(int64_t));
    for (uint32_t k = 0; k < d->n_chan; k++) c->chanSolverOf[k] = -1;
    c->channel = (ChannelStruct*)xcalloc(d->n_chan, sizeof(ChannelStruct));
    c->Gk = (double*)xcalloc(d->n_chan, sizeof(double));
    c->Ek = (double*)xcalloc(d->n_chan, sizeof(double));
    c->chanModel = (uint32_t*)xcalloc(d->n_chan, sizeof(uint32_t));
    c->chan2compt = (uint32_t*)xcalloc(d->n_chan, sizeof(uint32_t));
    c->chan2state = (uint32_t*)xcalloc(d->n_chan, sizeof(uint32_t));
    uint32_t nc = 0;
    for (uint32_t ic = 0; ic < n; ic++) {
        uint32_t m = c->compartmentId[ic];
        for (uint32_t k = 0; k < d->n_chan; k++) if (d->chan_compt[k] == m) {
            ChannelStruct* s = &c->channel[nc];
            c->Ek[nc] = d->chan_Ek[k];
            s->Gbar = d->chan_Gbar[k];
            s->Xpower = d->chan_Xpower[k]; s->Ypower = d->chan_Ypower[k]; s->Zpower = d->chan_Zpower[k];
            s->instant = d->chan_instant[k];
            s->modulation = d->chan_modulation[k];
            c->chan2state[nc] = (uint32_t)c->state.n;
            if (s->Xpower > 0.0) dpush(&c->state, d->chan_X[k]);
            if (s->Ypower > 0.0) dpush(&c->state, d->chan_Y[k]);
            if (s->Zpower > 0.0) dpush(&c->state, d->chan_Z[k]);
            c->chan2compt[nc] = ic;
            c->chanModel[nc] = k;
            c->chanSolverOf[k] = nc;
            c->channelCount[ic]++;
            nc++;
        }
    }
    c->nChan = nc;
    c->currentBoundary = (uint32_t*)xcalloc(n, sizeof(uint32_t));
    { uint32_t cum = 0; for (uint32_t ic = 0; ic < n; ic++) { cum += c->channelCount[ic]; c->currentBoundary[ic] = cum; } }

    /* readGates (hsolve/HSolveActiveSetup.cpp:237-250) */
    c->gateId = (int64_t*)xcalloc(3 * (size_t)nc, sizeof(int64_t));
    c->gCaDepend = (int*)xcalloc(3 * (size_t)nc, sizeof(int));
    for (uint32_t q = 0; q < nc; q++) {
        uint32_t k = c->chanModel[q];
        size_t first = c->nGateIds;
        if (d->chan_Xpower[k] > 0.0) c->gateId[c->nGateIds++] = d->chan_xgate[k];
        if (d->chan_Ypower[k] > 0.0) c->gateId[c->nGateIds++] = d->chan_ygate[k];
        if (d->chan_Zpower[k] > 0.0) c->gateId[c->nGateIds++] = d->chan_zgate[k];
        for (size_t g = first; g < c->nGateIds; g++) {
            if (c->gateId[g] < 0 || c->gateId[g] >= (int64_t)d->n_gate) FAIL("channel gate index out of range");
            c->gCaDepend[g] = 0;
        }
        if (d->chan_use_conc[k] && c->nGateIds > first) c->gCaDepend[c->nGateIds - 1] = 1;
    }

    /* readCalcium (hsolve/HSolveActiveSetup.cpp:252-337) */
    c->caCount = (uint32_t*)xcalloc(n, sizeof(uint32_t));
    c->caDependIndex = (int64_t*)xcalloc(nc + 1, sizeof(int64_t));
    int64_t* caTargetIndex = (int64_t*)xcalloc(nc + 1, sizeof(int64_t));
    int64_t* caConcIndex = (int64_t*)xcalloc(d->n_pool + 1, sizeof(int64_t));
    for (uint32_t p = 0; p < d->n_pool; p++) caConcIndex[p] = -1;
    c->caConc = (CaConcStruct*)xcalloc(d->n_pool + 1, sizeof(CaConcStruct));
    c->poolModel = (uint32_t*)xcalloc(d->n_pool + 1, sizeof(uint32_t));
    c->poolSolverOf = (int64_t*)xcalloc(d->n_pool + 1, sizeof(int64_t));
    for (uint32_t p = 0; p < d->n_pool; p++) c->poolSolverOf[p] = -1;
    c->externalCalcium = (double*)xcalloc(nc + 1, sizeof(double));
    size_t nTI = 0, nDI = 0;
    uint32_t ichan = 0;
    for (uint32_t ic = 0; ic < n; ++ic) {
        uint32_t chanBoundary = ichan + c->channelCount[ic];
        uint32_t nCa = c->nPool;
        for (; ichan < chanBoundary; ++ichan) {
            uint32_t k = c->chanModel[ichan];
            int64_t ids[2]; int nid = 0;
            int nTarget = d->chan_ca_target[k] >= 0;
            if (nTarget) ids[nid++] = d->chan_ca_target[k];
            else caTargetIndex[nTI++] = -1;
            int nDepend = d->chan_ca_depend[k] >= 0;
            if (nDepend) ids[nid++] = d->chan_ca_depend[k];
            else c->caDependIndex[nDI++] = -1;
            c->externalCalcium[ichan] = 0;
            for (int q = 0; q < nid; q++) {
                int64_t p = ids[q];
                if (p >= (int64_t)d->n_pool) FAIL("channel pool index out of range");
                if (caConcIndex[p] < 0) {
                    caConcIndex[p] = c->caCount[ic];
                    ++c->caCount[ic];
                    CaConcStruct* s = &c->caConc[c->nPool];
                    /* CaConcStruct(Ca, CaBasal, tau, B, ceiling, floor, dt):
                       setCa then setCaBasal leave c_ = Ca - CaBasal */
                    s->CaBasal = d->pool_CaBasal[p];
                    s->c = d->pool_Ca[p] - d->pool_CaBasal[p];
                    ca_setTauB(s, d->pool_tau[p], d->pool_B[p], dt);
                    s->ceiling = d->pool_ceiling[p];
                    s->floor_ = d->pool_floor[p];
                    c->poolModel[c->nPool] = (uint32_t)p;
                    c->poolSolverOf[p] = c->nPool;
                    c->nPool++;
                }
            }
            if (nTarget) caTargetIndex[nTI++] = caConcIndex[ids[0]] + nCa;
            if (nDepend) c->caDependIndex[nDI++] = caConcIndex[ids[nid - 1]];
        }
    }
    c->caTarget = (int64_t*)xcalloc(nc + 1, sizeof(int64_t));
    c->ca = (double*)xcalloc(c->nPool + 1, sizeof(double));
    c->caActivation = (double*)xcalloc(c->nPool + 1, sizeof(double));
    for (uint32_t q = 0; q < nc; ++q) c->caTarget[q] = caTargetIndex[q];
    free(caTargetIndex);
    free(caConcIndex);

    /* createLookupTables (hsolve/HSolveActiveSetup.cpp:339-526) */
    {
        int64_t* caSet = (int64_t*)xcalloc(c->nGateIds + 1, sizeof(int64_t));
        int64_t* vSet = (int64_t*)xcalloc(c->nGateIds + 1, sizeof(int64_t));
        size_t nca = 0, nv = 0;
        for (size_t g = 0; g < c->nGateIds; g++) {
            if (c->gCaDepend[g]) caSet[nca++] = c->gateId[g]; else vSet[nv++] = c->gateId[g];
        }
        qsort(caSet, nca, sizeof(int64_t), cmp_i64);
        qsort(vSet, nv, sizeof(int64_t), cmp_i64);
        size_t u = 0; for (size_t q = 0; q < nca; q++) if (!u || caSet[u - 1] != caSet[q]) caSet[u++] = caSet[q]; nca = u;
        u = 0; for (size_t q = 0; q < nv; q++) if (!u || vSet[u - 1] != vSet[q]) vSet[u++] = vSet[q]; nv = u;
        int64_t* species = (int64_t*)xcalloc(d->n_gate + 1, sizeof(int64_t));
        for (size_t q = 0; q < nca; q++) species[caSet[q]] = (int64_t)q;
        for (size_t q = 0; q < nv; q++) species[vSet[q]] = (int64_t)q;
        c->vMin = DBL_MAX; c->vMax = DBL_MIN; double vDx = DBL_MAX;
        c->caMin = DBL_MAX; c->caMax = DBL_MIN; double caDx = DBL_MAX;
        for (size_t q = 0; q < nca; q++) {
            const HsGateTable* g = &d->gate[caSet[q]];
            double dx = (g->max - g->min) / g->divs;
            if (g->min < c->caMin) c->caMin = g->min;
            if (g->max > c->caMax) c->caMax = g->max;
            if (dx < caDx) caDx = dx;
        }
        double caDiv = (c->caMax - c->caMin) / caDx;
        c->caDiv = (int)(caDiv + 0.5);
        for (size_t q = 0; q < nv; q++) {
            const HsGateTable* g = &d->gate[vSet[q]];
            double dx = (g->max - g->min) / g->divs;
            if (g->min < c->vMin) c->vMin = g->min;
            if (g->max > c->vMax) c->vMax = g->max;
            if (dx < vDx) vDx = dx;
        }
        double vDiv = (c->vMax - c->vMin) / vDx;
        c->vDiv = (int)(vDiv + 0.5);
        lt_init(&c->caTable, c->caMin, c->caMax, (uint32_t)c->caDiv, (uint32_t)nca);
        lt_init(&c->vTable, c->vMin, c->vMax, (uint32_t)c->vDiv, (uint32_t)nv);
        for (int pass = 0; pass < 2; pass++) {
            LookupTable* t = pass ? &c->vTable : &c->caTable;
            int64_t* set = pass ? vSet : caSet;
            size_t ns = pass ? nv : nca;
            double gmin = pass ? c->vMin : c->caMin, gmax = pass ? c->vMax : c->caMax;
            unsigned int gdivs = (unsigned int)(pass ? c->vDiv : c->caDiv);
            double gdx = (gmax - gmin) / gdivs;
            size_t gsize = (size_t)gdivs + 1;
            double* A = (double*)xcalloc(gsize, sizeof(double));
            double* B = (double*)xcalloc(gsize, sizeof(double));
            for (size_t q = 0; q < ns; q++) {
                const HsGateTable* g = &d->gate[set[q]];
                if (g->min == gmin && g->max == gmax && g->divs == gdivs) {
                    lt_addColumns(t, (int)q, g->A, g->B, (size_t)g->divs + 1);
                } else {
                    for (size_t i = 0; i < gsize; i++) gate_lookupBoth(g, gmin + gdx * i, &A[i], &B[i]);
                    lt_addColumns(t, (int)q, A, B, gsize);
                }
            }
            free(A); free(B);
        }
        c->column = (uint32_t*)xcalloc(c->nGateIds + 1, sizeof(uint32_t));
        for (size_t g = 0; g < c->nGateIds; g++) c->column[g] = 2 * (uint32_t)species[c->gateId[g]];
        free(species); free(caSet); free(vSet);
        uint32_t maxN = 0;
        for (uint32_t ic = 0; ic < n; ic++) if (c->caCount[ic] > maxN) maxN = c->caCount[ic];
        c->caRowComptSize = maxN;
        c->caRowCompt = (LookupRow*)xcalloc(maxN + 1, sizeof(LookupRow));
        c->caRow = (int64_t*)xcalloc(nc + 1, sizeof(int64_t));
        size_t zr = 0;
        for (uint32_t q = 0; q < nc; ++q)
            if (c->channel[q].Zpower > 0.0) c->caRow[zr++] = c->caDependIndex[q];
    }

    /* readSynapses: spikegens per compartment in Hines order */
    c->nSg = d->n_spikegen;
    c->sgLast = (double*)xcalloc(c->nSg + 1, sizeof(double));
    c->sgFired = (int*)xcalloc(c->nSg + 1, sizeof(int));
    c->sgComptHines = (uint32_t*)xcalloc(c->nSg + 1, sizeof(uint32_t));
    for (uint32_t k = 0; k < c->nSg; k++) {
        if (d->sg_compt[k] >= d->n_compt || c->hinesOf[d->sg_compt[k]] == UINT32_MAX) FAIL("spikegen compartment not in the tree");
        c->sgComptHines[k] = c->hinesOf[d->sg_compt[k]];
    }
    /* readExternalChannels */
    c->externalCurrent = (double*)xcalloc(2 * (size_t)n, sizeof(double));
    c->prevExtCurr = (double*)xcalloc(2 * (size_t)n, sizeof(double));

    /* external objects */
    c->c2dX = (double*)xcalloc(d->n_chan2d + 1, sizeof(double));
    c->c2dVm = (double*)xcalloc(d->n_chan2d + 1, sizeof(double));
    c->c2dConc1 = (double*)xcalloc(d->n_chan2d + 1, sizeof(double));
    c->c2dConc2 = (double*)xcalloc(d->n_chan2d + 1, sizeof(double));
    c->c2dGk = (double*)xcalloc(d->n_chan2d + 1, sizeof(double));
    c->c2dMod = (double*)xcalloc(d->n_chan2d + 1, sizeof(double));
    for (uint32_t k = 0; k < d->n_chan2d; k++) c->c2dMod[k] = d->c2d_modulation[k];
    c->synMod = (double*)xcalloc(d->n_syn + 1, sizeof(double));
    for (uint32_t k = 0; k < d->n_syn; k++) c->synMod[k] = d->syn_modulation[k];
    for (uint32_t k = 0; k < d->n_chan2d; k++) {
        if (c->hinesOf[d->c2d_compt[k]] == UINT32_MAX) FAIL("HHChannel2D compartment not in the tree");
        if (d->c2d_xgate[k] < 0 || d->c2d_xgate[k] >= (int32_t)d->n_gate2d) FAIL("HHChannel2D gate index out of range");
        if (d->c2d_conc1_pool[k] >= 0 && c->poolSolverOf[d->c2d_conc1_pool[k]] < 0) FAIL("HHChannel2D conc1 pool is not taken by the solver");
        if (d->c2d_conc2_pool[k] >= 0 && c->poolSolverOf[d->c2d_conc2_pool[k]] < 0) FAIL("HHChannel2D conc2 pool is not taken by the solver");
    }
    uint32_t ns = d->n_syn;
    c->synX = (double*)xcalloc(ns + 1, sizeof(double)); c->synY = (double*)xcalloc(ns + 1, sizeof(double));
    c->synAct = (double*)xcalloc(ns + 1, sizeof(double)); c->synGk = (double*)xcalloc(ns + 1, sizeof(double));
    c->synXc1 = (double*)xcalloc(ns + 1, sizeof(double)); c->synXc2 = (double*)xcalloc(ns + 1, sizeof(double));
    c->synYc1 = (double*)xcalloc(ns + 1, sizeof(double)); c->synYc2 = (double*)xcalloc(ns + 1, sizeof(double));
    c->synNorm = (double*)xcalloc(ns + 1, sizeof(double)); c->synDt = (double*)xcalloc(ns + 1, sizeof(double));
    for (uint32_t k = 0; k < ns; k++)
        if (c->hinesOf[d->syn_compt[k]] == UINT32_MAX) FAIL("SynChan compartment not in the tree");
    /* event lists sorted by (time, input order) per synchan */
    c->evOff = (uint32_t*)xcalloc(ns + 1, sizeof(uint32_t));
    c->evPtr = (uint32_t*)xcalloc(ns + 1, sizeof(uint32_t));
    c->evTime = (double*)xcalloc(d->n_event + 1, sizeof(double));
    c->evW = (double*)xcalloc(d->n_event + 1, sizeof(double));
    c->rtTime = (dvec*)xcalloc(ns + 1, sizeof(dvec));
    c->rtW = (dvec*)xcalloc(ns + 1, sizeof(dvec));
    c->rtHead = (uint32_t*)xcalloc(ns + 1, sizeof(uint32_t));
    for (uint32_t e = 0; e < d->n_event; e++) {
        if (d->ev_syn[e] >= ns) FAIL("event synchan index out of range");
        c->evOff[d->ev_syn[e] + 1]++;
    }
    for (uint32_t k = 0; k < ns; k++) c->evOff[k + 1] += c->evOff[k];
    {
        uint32_t* fill = (uint32_t*)xcalloc(ns + 1, sizeof(uint32_t));
        for (uint32_t e = 0; e < d->n_event; e++) {
            uint32_t k = d->ev_syn[e];
            uint32_t pos = c->evOff[k] + fill[k]++;
            /* insertion keeps (time, input order) */
            while (pos > c->evOff[k] && c->evTime[pos - 1] > d->ev_time[e]) {
                c->evTime[pos] = c->evTime[pos - 1]; c->evW[pos] = c->evW[pos - 1]; pos--;
            }
            c->evTime[pos] = d->ev_time[e]; c->evW[pos] = d->ev_weight[e];
        }
        free(fill);
    }
    for (uint32_t k = 0; k < d->n_stim; k++) {
        if (d->stim_compt[k] >= d->n_compt || c->hinesOf[d->stim_compt[k]] == UINT32_MAX) FAIL("stimulus compartment not in the tree");
        if (k && d->stim_step[k] < d->stim_step[k - 1]) FAIL("stimulus schedule not sorted by step");
    }
    {
        const char* e = dif_setup(c);
        if (e) FAIL(e);
    }
    return c;
#undef FAIL
}

/* ------------------------------------------------------------------ */
/* Interpol2D::innerLookup + interpolate (builtins/Interpol2D.cpp:508-592) */
static double interp2d(const HsGate2DTable* g, const double* T, double x, double y) {
    unsigned long nx = g->xdivs + 1, ny = g->ydivs + 1;
    if (x < g->xmin) x = g->xmin;
    if (x > g->xmax) x = g->xmax;
    if (y < g->ymin) y = g->ymin;
    if (y > g->ymax) y = g->ymax;
    double invDx = (double)g->xdivs / (g->xmax - g->xmin);
    double invDy = (double)g->ydivs / (g->ymax - g->ymin);
    int endX = 0, endY = 0;
    double z00 = 0.0, z01 = 0.0, z10 = 0.0, z11 = 0.0;
    double xv = (x - g->xmin) * invDx;
    unsigned long xi = (unsigned long)xv;
    if (xi >= nx) xi = nx - 1;
    if (xi == nx - 1) endX = 1;
    double xF = xv - xi;
    double yv = (y - g->ymin) * invDy;
    unsigned long yi = (unsigned long)yv;
    if (yi >= ny) yi = ny - 1;
    if (yi == ny - 1) endY = 1;
    double yF = yv - yi;
    double xFyF = xF * yF;
    z00 = T[xi * ny + yi];
    if (!endX) {
        z10 = T[(xi + 1) * ny + yi];
        if (!endY) { z11 = T[(xi + 1) * ny + yi + 1]; z01 = T[xi * ny + yi + 1]; }
    } else if (!endY) {
        z01 = T[xi * ny + yi + 1];
    }
    return z00 * (1 - xF - yF + xFyF) + z10 * (xF - xFyF) + z01 * (yF - xFyF) + z11 * xFyF;
}

/* HHChannel2D::dependency -> value: 0 Vm, 1 conc1, 2 conc2, -1 none */
static void dep_codes(int xindex, int* d0, int* d1) {
    switch (xindex) {
    case HS_DEP_VOLT: *d0 = 0; *d1 = -1; break;
    case HS_DEP_C1: *d0 = 1; *d1 = -1; break;
    case HS_DEP_C2: *d0 = 2; *d1 = -1; break;
    case HS_DEP_VOLT_C1: *d0 = 0; *d1 = 1; break;
    case HS_DEP_VOLT_C2: *d0 = 0; *d1 = 2; break;
    default: *d0 = 1; *d1 = 2; break;
    }
}
static double dep_value(int dep, double vm, double c1, double c2) {
    return dep == 0 ? vm : dep == 1 ? c1 : dep == 2 ? c2 : 0.0;
}

/* ------------------------------------------------------------------ */
/* HSolveActive::reinit (hsolve/HSolveActiveSetup.cpp:43-160) plus the
 * tick-1/4 objects' reinit (which run before tick 6). */
void orc_reinit(OrcCell* c, double clock_dt) {
    const HsCellDesc* d = c->d;
    uint32_t n = c->nCompt;
    c->dt = clock_dt;     /* HSolve::reinit: dt_ = p->dt */
    c->clockDt = clock_dt;
    c->nSteps = 0;
    c->stimPtr = 0;
    c->spikeGen.n = 0; c->spikeTime.n = 0;
    /* SimpleSynHandler::vReinit clears the queue; the events of the
       description are (re)queued afterwards. SynChan::vReinit. */
    for (uint32_t k = 0; k < d->n_syn; k++) {
        double dt = clock_dt;
        double tau1 = d->syn_tau1[k], tau2 = d->syn_tau2[k];
        c->evPtr[k] = c->evOff[k];
        c->rtTime[k].n = 0; c->rtW[k].n = 0; c->rtHead[k] = 0;
        c->synDt[k] = dt;
        c->synAct[k] = 0.0; c->synGk[k] = 0.0; c->synX[k] = 0.0; c->synY[k] = 0.0;
        c->synXc1[k] = tau1 * (1.0 - exp(-dt / tau1));
        c->synXc2[k] = exp(-dt / tau1);
        if (tau2 == 0.0) { c->synYc1[k] = 1.0; c->synYc2[k] = 0.0; }
        else { c->synYc1[k] = tau2 * (1.0 - exp(-dt / tau2)); c->synYc2[k] = exp(-dt / tau2); }
        double gbar = d->syn_Gbar[k];
        if (tau2 == 0.0) c->synNorm[k] = gbar;
        else if (tau1 == tau2) c->synNorm[k] = gbar * exp(1.0) / tau1;
        else {
            double tpeak = tau1 * tau2 * log(tau1 / tau2) / (tau1 - tau2);
            c->synNorm[k] = gbar * (tau1 - tau2) / (tau1 * tau2 * (exp(-tpeak / tau1) - exp(-tpeak / tau2)));
        }
    }
    for (uint32_t k = 0; k < d->n_chan2d; k++) { c->c2dX[k] = d->c2d_X[k]; c->c2dGk[k] = 0.0; }

    memset(c->externalCurrent, 0, 2 * (size_t)n * sizeof(double));
    for (uint32_t k = 0; k < c->nSg; k++) c->sgLast[k] = -d->sg_refractT[k];
    for (uint32_t ic = 0; ic < n; ++ic) c->V[ic] = c->initVm[ic];
    for (uint32_t p = 0; p < c->nPool; p++) c->caActivation[p] = 0.0;
    for (uint32_t p = 0; p < c->nPool; p++) { c->caConc[p].c = 0.0; c->ca[p] = c->caConc[p].CaBasal; }
    /* tick 1 reinits before the solver's tick 6: the shells' concentrations
       reach the channels' external calcium the gates start from */
    dif_reinit(c);
    /* reinitChannels */
    uint32_t ichan = 0, ica = 0, icol = 0, izr = 0;
    size_t istate = 0;
    LookupRow vRow, dRow;
    for (uint32_t ic = 0; ic < n; ++ic) {
        lt_row(&c->vTable, c->V[ic], &vRow);
        uint32_t caBoundary = ica + c->caCount[ic];
        uint32_t rc = 0;
        for (; ica < caBoundary; ++ica) lt_row(&c->caTable, c->ca[ica], &c->caRowCompt[rc++]);
        uint32_t chanBoundary = ichan + c->channelCount[ic];
        for (; ichan < chanBoundary; ++ichan) {
            ChannelStruct* ch = &c->channel[ichan];
            double C1, C2;
            if (c->caTable.nColumns) lt_row(&c->caTable, c->externalCalcium[ichan], &dRow);
            if (ch->Xpower > 0.0) { lt_lookup(&c->vTable, c->column[icol], &vRow, &C1, &C2); c->state.v[istate] = C1 / C2; ++icol, ++istate; }
            if (ch->Ypower > 0.0) { lt_lookup(&c->vTable, c->column[icol], &vRow, &C1, &C2); c->state.v[istate] = C1 / C2; ++icol, ++istate; }
            if (ch->Zpower > 0.0) {
                int64_t cr = c->caRow[izr];
                if (cr >= 0) lt_lookup(&c->caTable, c->column[icol], &c->caRowCompt[cr], &C1, &C2);
                else if (c->externalCalcium[ichan] > 0) lt_lookup(&c->caTable, c->column[icol], &dRow, &C1, &C2);
                else lt_lookup(&c->vTable, c->column[icol], &vRow, &C1, &C2);
                c->state.v[istate] = C1 / C2;
                ++icol, ++istate, ++izr;
            }
        }
    }
    /* sendValues: tick-4 consumers get V and Ca */
    for (uint32_t k = 0; k < d->n_chan2d; k++) {
        c->c2dVm[k] = c->V[c->hinesOf[d->c2d_compt[k]]];
        c->c2dConc1[k] = d->c2d_conc1_pool[k] >= 0 ? c->ca[c->poolSolverOf[d->c2d_conc1_pool[k]]] : 0.0;
        c->c2dConc2[k] = d->c2d_conc2_pool[k] >= 0 ? c->ca[c->poolSolverOf[d->c2d_conc2_pool[k]]] : 0.0;
    }
}

/* HSolveActive::advanceChannels (hsolve/HSolveActive.cpp:218-332) */
/* Conditioning probe (not the reference's arithmetic): the trapezoidal gate
   step written as x + (dt C1 - 2 h x)/(1 + h), h = dt/2 C2, with the
   increment computed in FP32 and added to the FP64 state -- the precision a
   mixed-precision solver gives its gates.  A cell whose trajectory leaves a
   tolerance under this alone is ill-conditioned at that tolerance for any
   solver with FP32 gating. */
static double gateIncrementF32(double x, double C1, double C2, double dt) {
    const float c1 = (float)C1, c2 = (float)C2, xf = (float)x, dtf = (float)dt;
    const float h = 0.5f * dtf * c2;
    const float inc = (dtf * c1 - 2.0f * h * xf) / (1.0f + h);
    return (double)inc;
}

static void advanceChannels(OrcCell* c, double dt) {
    uint32_t n = c->nCompt;
    uint32_t ichan = 0, ica = 0, icol = 0, izr = 0;
    size_t istate = 0;
    LookupRow vRow, dRow;
    double* state = c->state.v;
    for (uint32_t ic = 0; ic < n; ++ic) {
        lt_row(&c->vTable, c->V[ic], &vRow);
        uint32_t caBoundary = ica + c->caCount[ic];
        uint32_t rc = 0;
        for (; ica < caBoundary; ++ica) lt_row(&c->caTable, c->ca[ica], &c->caRowCompt[rc++]);
        uint32_t chanBoundary = ichan + c->channelCount[ic];
        for (; ichan < chanBoundary; ++ichan) {
            ChannelStruct* ch = &c->channel[ichan];
            double C1, C2;
            if (c->caTable.nColumns) lt_row(&c->caTable, c->externalCalcium[ichan], &dRow);
            if (ch->Xpower > 0.0) {
                lt_lookup(&c->vTable, c->column[icol], &vRow, &C1, &C2);
                if (ch->instant & 1) state[istate] = C1 / C2;
                else if (c->f32GateIncrements) state[istate] += gateIncrementF32(state[istate], C1, C2, dt);
                else { double temp = 1.0 + dt / 2.0 * C2; state[istate] = (state[istate] * (2.0 - temp) + dt * C1) / temp; }
                ++icol, ++istate;
            }
            if (ch->Ypower > 0.0) {
                lt_lookup(&c->vTable, c->column[icol], &vRow, &C1, &C2);
                if (ch->instant & 2) state[istate] = C1 / C2;
                else if (c->f32GateIncrements) state[istate] += gateIncrementF32(state[istate], C1, C2, dt);
                else { double temp = 1.0 + dt / 2.0 * C2; state[istate] = (state[istate] * (2.0 - temp) + dt * C1) / temp; }
                ++icol, ++istate;
            }
            if (ch->Zpower > 0.0) {
                int64_t cr = c->caRow[izr];
                if (cr >= 0) lt_lookup(&c->caTable, c->column[icol], &c->caRowCompt[cr], &C1, &C2);
                else if (c->externalCalcium[ichan] > 0) lt_lookup(&c->caTable, c->column[icol], &dRow, &C1, &C2);
                else lt_lookup(&c->vTable, c->column[icol], &vRow, &C1, &C2);
                if (ch->instant & 4) state[istate] = C1 / C2;
                else if (c->f32GateIncrements) state[istate] += gateIncrementF32(state[istate], C1, C2, dt);
                else { double temp = 1.0 + dt / 2.0 * C2; state[istate] = (state[istate] * (2.0 - temp) + dt * C1) / temp; }
                ++icol, ++istate, ++izr;
            }
        }
    }
}

/* calculateChannelCurrents + ChannelStruct::process */
static void calculateChannelCurrents(OrcCell* c) {
    size_t istate = 0;
    for (uint32_t q = 0; q < c->nChan; q++) {
        ChannelStruct* ch = &c->channel[q];
        double fraction = ch->modulation;
        if (ch->Xpower > 0.0) fraction *= takePower(c->state.v[istate++], ch->Xpower);
        if (ch->Ypower > 0.0) fraction *= takePower(c->state.v[istate++], ch->Ypower);
        if (ch->Zpower > 0.0) fraction *= takePower(c->state.v[istate++], ch->Zpower);
        c->Gk[q] = ch->Gbar * fraction;
    }
}

/* HSolveActive::updateMatrix (hsolve/HSolveActive.cpp:85-151) */
static void updateMatrixActive(OrcCell* c) {
    uint32_t n = c->nCompt;
    if (c->H) memcpy(c->mem + 4 * (size_t)n, c->HJCopy, c->H * sizeof(double));
    uint32_t icur = 0;
    for (uint32_t ic = 0; ic < n; ++ic) {
        double GkSum = 0.0, GkEkSum = 0.0;
        for (; icur < c->currentBoundary[ic]; ++icur) {
            GkSum += c->Gk[icur];
            GkEkSum += c->Gk[icur] * c->Ek[icur];
        }
        HS(4 * ic) = HS(4 * ic + 2) + GkSum;
        HS(4 * ic + 3) = c->V[ic] * c->CmByDt[ic] + c->EmByRm[ic] + GkEkSum;
    }
    for (uint32_t ic = 0; ic < n; ++ic) if (c->injPresent[ic]) {
        HS(4 * ic + 3) += c->injectVarying[ic] + c->injectBasal[ic];
        c->injectVarying[ic] = 0.0;
    }
    for (uint32_t ic = 0; ic < n; ++ic) {
        HS(4 * ic) += c->externalCurrent[2 * ic];
        HS(4 * ic + 3) += c->externalCurrent[2 * ic + 1];
    }
    c->stage = 0;
}

/* HSolveActive::advanceCalcium (hsolve/HSolveActive.cpp:153-216) */
static void advanceCalcium(OrcCell* c) {
    uint32_t n = c->nCompt;
    const double* VMid = c->mem + 4 * (size_t)n + c->H;
    uint32_t icur = 0;
    for (uint32_t ic = 0; ic < n; ++ic) {
        for (; icur < c->currentBoundary[ic]; ++icur) {
            if (c->caTarget[icur] >= 0) {
                double v = c->caAdvance == 1 ? VMid[ic] : (2 * VMid[ic] - c->V[ic]);
                c->caActivation[c->caTarget[icur]] += c->Gk[icur] * (c->Ek[icur] - v);
            }
        }
    }
    for (uint32_t p = 0; p < c->nPool; p++) c->ca[p] = ca_process(&c->caConc[p], c->caActivation[p]);
    for (uint32_t p = 0; p < c->nPool; p++) c->caActivation[p] = 0.0;
}

void orc_step(OrcCell* c, uint32_t nsteps) {
    const HsCellDesc* d = c->d;
    uint32_t n = c->nCompt;
    for (uint32_t s = 0; s < nsteps; s++) {
        double dt = c->clockDt;
        double currTime = dt * (double)(c->nSteps + 1);   /* Clock: dt_ * endStep */
        /* tick 0: basal-inject schedule */
        while (c->stimPtr < d->n_stim && d->stim_step[c->stimPtr] <= c->nSteps) {
            uint32_t h = c->hinesOf[d->stim_compt[c->stimPtr]];
            c->injPresent[h] = 1;
            c->injectBasal[h] = d->stim_value[c->stimPtr];
            c->stimPtr++;
        }
        /* tick 1: SimpleSynHandler -> SynChan::activation */
        for (uint32_t k = 0; k < d->n_syn; k++) {
            double activation = 0.0;
            const dvec* rt = &c->rtTime[k];
            for (;;) {
                int desc = c->evPtr[k] < c->evOff[k + 1] && c->evTime[c->evPtr[k]] <= currTime;
                int run = c->rtHead[k] < rt->n && rt->v[c->rtHead[k]] <= currTime;
                if (desc && (!run || c->evTime[c->evPtr[k]] <= rt->v[c->rtHead[k]])) {
                    activation += c->evW[c->evPtr[k]] / dt;
                    c->evPtr[k]++;
                } else if (run) {
                    activation += c->rtW[k].v[c->rtHead[k]] / dt;
                    c->rtHead[k]++;
                } else {
                    break;
                }
            }
            if (activation != 0.0) c->synAct[k] += activation;
        }
        /* tick 1: DifShells, DifBuffers, MMPumps */
        dif_process(c, dt);
        /* tick 4: each object -> addGkEk.  The reference's clock sends the
           HHChannel2Ds in creation order and then the SynChans in reverse
           creation order (scheduling/Clock.cpp:764-774 over the proc4 message
           list); the order only matters for the rounding of the sums. */
        for (uint32_t k = 0; k < d->n_chan2d; k++) {
            const HsGate2DTable* g = &d->gate2d[d->c2d_xgate[k]];
            double g_ = d->c2d_Gbar[k];
            if (d->c2d_Xpower[k] > 0) {
                int d0, d1;
                dep_codes(d->c2d_xindex[k], &d0, &d1);
                double x = dep_value(d0, c->c2dVm[k], c->c2dConc1[k], c->c2dConc2[k]);
                double y = dep_value(d1, c->c2dVm[k], c->c2dConc1[k], c->c2dConc2[k]);
                double A = interp2d(g, g->A, x, y);
                double B = interp2d(g, g->B, x, y);
                if (d->c2d_instant[k] & 1) c->c2dX[k] = A / B;
                else if (B > 1.0e-10) { double e = exp(-B * dt); c->c2dX[k] = c->c2dX[k] * e + (A / B) * (1 - e); }
                else c->c2dX[k] = c->c2dX[k] + A * dt;
                g_ *= takePower(c->c2dX[k], d->c2d_Xpower[k]);
            }
            c->c2dGk[k] = g_ * c->c2dMod[k];
            uint32_t h = c->hinesOf[d->c2d_compt[k]];
            c->externalCurrent[2 * h] += c->c2dGk[k];
            c->externalCurrent[2 * h + 1] += c->c2dGk[k] * d->c2d_Ek[k];
        }
        for (uint32_t kk = d->n_syn; kk-- > 0;) {
            uint32_t k = kk;
            c->synX[k] = c->synAct[k] * c->synXc1[k] + c->synX[k] * c->synXc2[k];
            c->synY[k] = c->synX[k] * c->synYc1[k] + c->synY[k] * c->synYc2[k];
            c->synAct[k] = 0.0;
            c->synGk[k] = c->synY[k] * c->synNorm[k] * c->synMod[k];
            uint32_t h = c->hinesOf[d->syn_compt[k]];
            c->externalCurrent[2 * h] += c->synGk[k];
            c->externalCurrent[2 * h + 1] += c->synGk[k] * d->syn_Ek[k];
        }
        /* tick 6: HSolveActive::step */
        if (n > 0) {
            advanceChannels(c, dt);
            calculateChannelCurrents(c);
            updateMatrixActive(c);
            orc_forward(c);
            orc_backward(c);
            advanceCalcium(c);
            dif_send_ik(c);
            /* sendValues -> tick-4 consumers of the next step */
            for (uint32_t k = 0; k < d->n_chan2d; k++) {
                c->c2dVm[k] = c->V[c->hinesOf[d->c2d_compt[k]]];
                if (d->c2d_conc1_pool[k] >= 0) c->c2dConc1[k] = c->ca[c->poolSolverOf[d->c2d_conc1_pool[k]]];
                if (d->c2d_conc2_pool[k] >= 0) c->c2dConc2[k] = c->ca[c->poolSolverOf[d->c2d_conc2_pool[k]]];
            }
            /* sendSpikes: SpikeGen::handleVm + process at currTime */
            for (uint32_t k = 0; k < c->nSg; k++) {
                double V = c->V[c->sgComptHines[k]];
                if (V > d->sg_threshold[k]) {
                    if ((currTime + dt / 2.0) >= (c->sgLast[k] + d->sg_refractT[k])) {
                        if (!(d->sg_edge[k] && c->sgFired[k])) {
                            ipush(&c->spikeGen, k);
                            dpush(&c->spikeTime, currTime);
                            c->sgLast[k] = currTime;
                            c->sgFired[k] = 1;
                        }
                    }
                } else {
                    c->sgFired[k] = 0;
                }
            }
            memcpy(c->prevExtCurr, c->externalCurrent, 2 * (size_t)n * sizeof(double));
            memset(c->externalCurrent, 0, 2 * (size_t)n * sizeof(double));
        }
        c->nSteps++;
    }
}

/* ------------------------------------------------------------------ */
uint32_t orc_n_compt(const OrcCell* c) { return c->nCompt; }
uint32_t orc_n_pool(const OrcCell* c) { return c->nPool; }
uint32_t orc_n_state(const OrcCell* c) { return (uint32_t)c->state.n; }
uint32_t orc_hines_index(const OrcCell* c, uint32_t m) { return c->hinesOf[m]; }
uint32_t orc_model_index(const OrcCell* c, uint32_t h) { return c->compartmentId[h]; }
void orc_set_ca_advance(OrcCell* c, int a) { c->caAdvance = a; }
void orc_set_f32_gate_increments(OrcCell* c, int on) { c->f32GateIncrements = on != 0; }

void orc_read_vm(const OrcCell* c, double* out) {
    for (uint32_t m = 0; m < c->d->n_compt; m++)
        out[m] = c->hinesOf[m] == UINT32_MAX ? NAN : c->V[c->hinesOf[m]];
}
void orc_read_ca(const OrcCell* c, double* out) {
    for (uint32_t p = 0; p < c->d->n_pool; p++)
        out[p] = c->poolSolverOf[p] < 0 ? NAN : c->ca[c->poolSolverOf[p]];
}
void orc_read_state(const OrcCell* c, double* out) { memcpy(out, c->state.v, c->state.n * sizeof(double)); }
uint32_t orc_read_spikes(const OrcCell* c, uint32_t* gen, double* t, uint32_t cap) {
    for (uint32_t k = 0; k < c->spikeGen.n && k < cap; k++) { gen[k] = (uint32_t)c->spikeGen.v[k]; t[k] = c->spikeTime.v[k]; }
    return (uint32_t)c->spikeGen.n;
}
void orc_table_grid(const OrcCell* c, double* g) {
    g[0] = c->vMin; g[1] = c->vMax; g[2] = c->vDiv; g[3] = c->caMin; g[4] = c->caMax; g[5] = c->caDiv;
}

/* state index of gate `which` (0 X, 1 Y, 2 Z) of solver channel q, or -1 */
static int64_t gate_state(const OrcCell* c, uint32_t q, int which) {
    const ChannelStruct* ch = &c->channel[q];
    double p[3] = {ch->Xpower, ch->Ypower, ch->Zpower};
    if (p[which] == 0.0) return -1;
    int64_t s = c->chan2state[q];
    for (int w = 0; w < which; w++) if (p[w] > 0.0) s++;
    return s;
}

int orc_get_field(const OrcCell* c, int kind, int field, uint32_t index, double* out) {
    if (kind == HS_KIND_COMPT) {
        if (index >= c->d->n_compt || c->hinesOf[index] == UINT32_MAX) return HS_EINVAL;
        uint32_t i = c->hinesOf[index];
        switch (field) {
        case HS_F_VM: *out = c->V[i]; return 0;
        case HS_F_CM: *out = c->Cm[i]; return 0;
        case HS_F_EM: *out = c->Em[i]; return 0;
        case HS_F_RM: *out = c->Rm[i]; return 0;
        case HS_F_RA: *out = c->Ra[i]; return 0;
        case HS_F_INITVM: *out = c->initVm[i]; return 0;
        case HS_F_INJECT: *out = c->injPresent[i] ? c->injectBasal[i] : 0.0; return 0;
        case HS_F_IM: {
            double Im = c->EmByRm[i] - c->V[i] / c->Rm[i];
            uint32_t b = i == 0 ? 0 : c->currentBoundary[i - 1];
            for (; b < c->currentBoundary[i]; ++b) Im += (c->Ek[b] - c->V[i]) * c->Gk[b];
            Im += c->prevExtCurr[2 * i + 1] - c->prevExtCurr[2 * i] * c->V[i];
            *out = Im; return 0;
        }
        }
        return HS_EINVAL;
    }
    if (kind == HS_KIND_CHAN) {
        if (index >= c->d->n_chan || c->chanSolverOf[index] < 0) return HS_EINVAL;
        uint32_t q = (uint32_t)c->chanSolverOf[index];
        int64_t s;
        switch (field) {
        case HS_F_GBAR: *out = c->channel[q].Gbar; return 0;
        case HS_F_EK: *out = c->Ek[q]; return 0;
        case HS_F_GK: *out = c->Gk[q]; return 0;
        case HS_F_IK: *out = (c->Ek[q] - c->V[c->chan2compt[q]]) * c->Gk[q]; return 0;
        case HS_F_X: s = gate_state(c, q, 0); *out = s < 0 ? 0.0 : c->state.v[s]; return 0;
        case HS_F_Y: s = gate_state(c, q, 1); *out = s < 0 ? 0.0 : c->state.v[s]; return 0;
        case HS_F_Z: s = gate_state(c, q, 2); *out = s < 0 ? 0.0 : c->state.v[s]; return 0;
        case HS_F_INSTANT: *out = c->channel[q].instant; return 0;
        case HS_F_MODULATION: *out = c->channel[q].modulation; return 0;
        }
        return HS_EINVAL;
    }
    if (kind == HS_KIND_POOL) {
        if (index >= c->d->n_pool || c->poolSolverOf[index] < 0) return HS_EINVAL;
        uint32_t p = (uint32_t)c->poolSolverOf[index];
        switch (field) {
        case HS_F_CA: *out = c->ca[p]; return 0;
        case HS_F_CABASAL: *out = c->caConc[p].CaBasal; return 0;
        case HS_F_CEILING: *out = c->caConc[p].ceiling; return 0;
        case HS_F_FLOOR: *out = c->caConc[p].floor_; return 0;
        }
        return HS_EINVAL;
    }
    if (kind == HS_KIND_CHAN2D) {
        if (index >= c->d->n_chan2d) return HS_EINVAL;
        if (field == HS_F_X) { *out = c->c2dX[index]; return 0; }
        if (field == HS_F_GK) { *out = c->c2dGk[index]; return 0; }
        return HS_EINVAL;
    }
    if (kind == HS_KIND_SYNCHAN) {
        if (index >= c->d->n_syn) return HS_EINVAL;
        if (field == HS_F_GK) { *out = c->synGk[index]; return 0; }
        if (field == HS_F_X) { *out = c->synX[index]; return 0; }
        if (field == HS_F_Y) { *out = c->synY[index]; return 0; }
        return HS_EINVAL;
    }
    return HS_EINVAL;
}

int orc_set_field(OrcCell* c, int kind, int field, uint32_t index, double value) {
    if (kind == HS_KIND_COMPT) {
        if (index >= c->d->n_compt || c->hinesOf[index] == UINT32_MAX) return HS_EINVAL;
        uint32_t i = c->hinesOf[index];
        switch (field) {
        case HS_F_VM: c->V[i] = value; return 0;
        case HS_F_CM: c->Cm[i] = value; c->CmByDt[i] = 2.0 * value / c->dt; return 0;
        case HS_F_EM: c->Em[i] = value; c->EmByRm[i] = value / c->Rm[i]; return 0;
        case HS_F_RM: c->Rm[i] = value; c->EmByRm[i] = c->Em[i] / value; return 0;
        case HS_F_RA: c->Ra[i] = value; return 0;
        case HS_F_INITVM: c->initVm[i] = value; return 0;
        case HS_F_INJECT: c->injPresent[i] = 1; c->injectBasal[i] = value; return 0;
        }
        return HS_EINVAL;
    }
    if (kind == HS_KIND_CHAN) {
        if (index >= c->d->n_chan || c->chanSolverOf[index] < 0) return HS_EINVAL;
        uint32_t q = (uint32_t)c->chanSolverOf[index];
        int64_t s;
        switch (field) {
        case HS_F_GBAR: c->channel[q].Gbar = value; return 0;
        case HS_F_EK: c->Ek[q] = value; return 0;
        case HS_F_GK: c->Gk[q] = value; return 0;
        case HS_F_X: s = gate_state(c, q, 0); if (s >= 0) c->state.v[s] = value; return 0;
        case HS_F_Y: s = gate_state(c, q, 1); if (s >= 0) c->state.v[s] = value; return 0;
        case HS_F_Z: s = gate_state(c, q, 2); if (s >= 0) c->state.v[s] = value; return 0;
        case HS_F_INSTANT: c->channel[q].instant = (int)value; return 0;
        case HS_F_MODULATION: if (value > 0.0) c->channel[q].modulation = value; return 0;
        }
        return HS_EINVAL;
    }
    /* HHChannel2D and SynChan stay outside the solver: their own modulation
     * field, set as given (ChanCommon::vSetModulation, biophysics/ChanCommon.cpp:46-49) */
    if (kind == HS_KIND_CHAN2D) {
        if (index >= c->d->n_chan2d) return HS_EINVAL;
        if (field == HS_F_MODULATION) { c->c2dMod[index] = value; return 0; }
        return HS_EINVAL;
    }
    if (kind == HS_KIND_SYNCHAN) {
        if (index >= c->d->n_syn) return HS_EINVAL;
        if (field == HS_F_MODULATION) { c->synMod[index] = value; return 0; }
        return HS_EINVAL;
    }
    if (kind == HS_KIND_POOL) {
        if (index >= c->d->n_pool || c->poolSolverOf[index] < 0) return HS_EINVAL;
        uint32_t p = (uint32_t)c->poolSolverOf[index];
        CaConcStruct* s = &c->caConc[p];
        switch (field) {
        case HS_F_CA: c->ca[p] = value; s->c = value - s->CaBasal; return 0;
        case HS_F_CABASAL: s->c += s->CaBasal - value; s->CaBasal = value; return 0;
        case HS_F_CEILING: s->ceiling = value; return 0;
        case HS_F_FLOOR: s->floor_ = value; return 0;
        }
        return HS_EINVAL;
    }
    return HS_EINVAL;
}

/* Message destinations of the solver, model indices (hsolve/HSolveInterface.cpp).
 * HSolve::addInject (:213-219): injectVarying += value (the map entry is made
 * if absent); consumed and zeroed by the next updateMatrix. */
int orc_add_inject(OrcCell* c, uint32_t compt, double value) {
    if (compt >= c->d->n_compt || c->hinesOf[compt] == UINT32_MAX) return HS_EINVAL;
    uint32_t i = c->hinesOf[compt];
    c->injPresent[i] = 1;
    c->injectVarying[i] += value;
    return 0;
}

/* HSolve::addGkEk (:247-252): externalCurrent[2i] += Gk, [2i+1] += Gk Ek. */
int orc_add_gkek(OrcCell* c, uint32_t compt, double Gk, double Ek) {
    if (compt >= c->d->n_compt || c->hinesOf[compt] == UINT32_MAX) return HS_EINVAL;
    uint32_t i = c->hinesOf[compt];
    c->externalCurrent[2 * i] += Gk;
    c->externalCurrent[2 * i + 1] += Gk * Ek;
    return 0;
}

/* HSolve::addConc (:254-259): externalCalcium[channel] = conc. */
int orc_add_conc(OrcCell* c, uint32_t chan, double conc) {
    if (chan >= c->d->n_chan || c->chanSolverOf[chan] < 0) return HS_EINVAL;
    c->externalCalcium[c->chanSolverOf[chan]] = conc;
    return 0;
}

/* HSolve::iCa (:469-480): caActivation[pool] += iCa. */
int orc_add_ica(OrcCell* c, uint32_t pool, double ica) {
    if (pool >= c->d->n_pool || c->poolSolverOf[pool] < 0) return HS_EINVAL;
    c->caActivation[c->poolSolverOf[pool]] += ica;
    return 0;
}

/* SimpleSynHandler::addSpike (synapse/SimpleSynHandler.cpp:86-90): the event
   joins the synchan's queue behind every queued event with time <= its own
   (the caller has added the synapse delay, synapse/Synapse.cpp:104-113). */
int orc_push_event(OrcCell* c, uint32_t syn, double time, double weight) {
    if (!c->d || syn >= c->d->n_syn || time != time) return HS_EINVAL;
    dvec* t = &c->rtTime[syn];
    dvec* w = &c->rtW[syn];
    if (c->rtHead[syn] == t->n) { t->n = 0; w->n = 0; c->rtHead[syn] = 0; }
    dpush(t, time);
    dpush(w, weight);
    size_t pos = t->n - 1;
    while (pos > c->rtHead[syn] && t->v[pos - 1] > time) {
        t->v[pos] = t->v[pos - 1]; w->v[pos] = w->v[pos - 1]; pos--;
    }
    t->v[pos] = time; w->v[pos] = weight;
    return 0;
}

void orc_read_dif(const OrcCell* c, double* out) {
    for (uint32_t k = 0; k < c->dif.n; k++) {
        int kind = c->d->dif_kind[k];
        out[k] = kind == HS_DIF_SHELL ? c->dif.C[k] : kind == HS_DIF_BUFFER ? c->dif.bFree[k] : 0.0;
    }
}

void orc_destroy(OrcCell* c) {
    if (!c) return;
    {
        DifObjs* o = &c->dif;
        double* arrs[] = {o->C, o->prevC, o->dC, o->Cm, o->bFree, o->bBound, o->prevFree, o->Af, o->Bf,
                          o->act, o->vol, o->outerA, o->innerA};
        for (size_t a = 0; a < sizeof(arrs) / sizeof(arrs[0]); a++) free(arrs[a]);
        free(o->off); free(o->dst); free(o->ikOff); free(o->ikDst);
    }
    free(c->compartmentId); free(c->hinesOf); free(c->V); free(c->CmByDt); free(c->EmByRm);
    free(c->injPresent); free(c->injectVarying); free(c->injectBasal);
    free(c->childOff); free(c->childIdx); free(c->Ra); free(c->Rm); free(c->Cm); free(c->Em); free(c->initVm);
    free(c->mem); free(c->HJCopy); free(c->Ga); free(c->junction); free(c->groupOff); free(c->groupIdx);
    free(c->groupNumber); free(c->operandBase); free(c->operand.v); free(c->backOperand.v);
    free(c->channel); free(c->Gk); free(c->Ek); free(c->chanModel); free(c->chanSolverOf);
    free(c->channelCount); free(c->currentBoundary); free(c->chan2compt); free(c->chan2state);
    free(c->state.v); free(c->gCaDepend); free(c->gateId);
    free(c->caConc); free(c->ca); free(c->caActivation); free(c->caTarget); free(c->caCount);
    free(c->caDependIndex); free(c->column); free(c->caRowCompt); free(c->caRow);
    free(c->externalCurrent); free(c->prevExtCurr); free(c->externalCalcium);
    free(c->poolModel); free(c->poolSolverOf);
    free(c->vTable.table); free(c->caTable.table);
    free(c->c2dX); free(c->c2dVm); free(c->c2dConc1); free(c->c2dConc2); free(c->c2dGk);
    free(c->c2dMod); free(c->synMod);
    free(c->synX); free(c->synY); free(c->synAct); free(c->synGk);
    free(c->synXc1); free(c->synXc2); free(c->synYc1); free(c->synYc2); free(c->synNorm); free(c->synDt);
    free(c->evOff); free(c->evTime); free(c->evW); free(c->evPtr);
    if (c->rtTime)
        for (uint32_t k = 0; k < c->d->n_syn; k++) { free(c->rtTime[k].v); free(c->rtW[k].v); }
    free(c->rtTime); free(c->rtW); free(c->rtHead);
    free(c->sgLast); free(c->sgFired); free(c->sgComptHines);
    free(c->spikeGen.v); free(c->spikeTime.v);
    free(c);
}
