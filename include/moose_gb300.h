/*
 * moose_gb300.h -- C ABI of the GB300 (sm_103a) HSolve.
 *
 * A drop-in for MOOSE's Hines solver (`HSolve`, reference `hsolve/HSolve.h:20`)
 * and for the per-step work of `HSolveActive::step`
 * (`hsolve/HSolveActive.cpp:45-66`).  The MOOSE side (an `HSolve` C++ class
 * registered under the same Cinfo name, fields and zombie classes) reads the
 * model once at setup, exactly as `HSolveActive::setup` does
 * (`hsolve/HSolveActiveSetup.cpp:17-41`), fills an `HsCellDesc`, and from then
 * on calls only the functions below.  No C++ types, exceptions or torch types
 * cross this boundary: plain pointers, sizes and `int` status codes.
 *
 * Conventions
 *  - Every function returns an HS_* status; 0 is success.  On failure the
 *    message is available from hs_last_error().
 *  - Indices are "model indices": positions in the arrays of the HsCellDesc
 *    the solver was created from (MOOSE's Id -> index map of
 *    `HSolve::localIndex`, `hsolve/HSolveInterface.cpp:23-36`, becomes the
 *    caller's own Id -> model-index map).
 *  - All quantities are SI, as in MOOSE (V, ohm, F, S, A, s, mM).
 */
#ifndef MOOSE_GB300_H
#define MOOSE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ */
/* Status codes (reference: `cerr` + early return, `hsolve/HSolve.cpp:409-434`,
 * and `assert` on unknown Ids, `hsolve/HSolveInterface.cpp:33`).        */
#define HS_OK        0
#define HS_EINVAL    1   /* bad argument, index or model                 */
#define HS_EDEVICE   2   /* CUDA error                                   */
#define HS_ENOMEM    3   /* host or device allocation failed             */
#define HS_ETIMEOUT  4   /* a bounded device wait gave up                */
#define HS_ESTATE    5   /* call not valid in the current state          */
#define HS_ENOTSUP   6   /* feature not supported by this build          */
#define HS_ECAPACITY 7   /* request larger than a fixed capacity         */

/* Precision of the per-step arithmetic. */
#define HS_PREC_FP64  0  /* every operation in FP64, reference order      */
#define HS_PREC_MIXED 1  /* FP32 gates/tables/synapses, FP64 matrix+solve */

/* ------------------------------------------------------------------ */
/* Model description.  One HsCellDesc describes what `HSolveActive::setup`
 * reads from the MOOSE object graph for one cell.                      */

/* An HHGate rate table (`biophysics/HHGate.cpp:539-620`): A = alpha and
 * B = alpha+beta sampled at min + i*(max-min)/divs, i = 0..divs.        */
typedef struct HsGateTable {
    double min;
    double max;
    uint32_t divs;
    const double* A;          /* divs+1 entries */
    const double* B;          /* divs+1 entries */
} HsGateTable;

/* An HHGate2D table pair (`builtins/Interpol2D.cpp`): entry [ix][iy] at
 * A[ix*(ydivs+1)+iy], x = xmin + ix*(xmax-xmin)/xdivs, same for y.      */
typedef struct HsGate2DTable {
    double xmin, xmax;
    double ymin, ymax;
    uint32_t xdivs, ydivs;
    const double* A;          /* (xdivs+1)*(ydivs+1) entries */
    const double* B;
} HsGate2DTable;

/* HHChannel2D index codes (`biophysics/HHChannel2D.cpp` `dependency`). */
#define HS_DEP_VOLT      0    /* "VOLT_INDEX"    */
#define HS_DEP_C1        1    /* "C1_INDEX"      */
#define HS_DEP_C2        2    /* "C2_INDEX"      */
#define HS_DEP_VOLT_C1   3    /* "VOLT_C1_INDEX" */
#define HS_DEP_VOLT_C2   4    /* "VOLT_C2_INDEX" */
#define HS_DEP_C1_C2     5    /* "C1_C2_INDEX"   */

typedef struct HsCellDesc {
    /* Compartments.  `parent[i]` is the morphological parent (the source of
     * the message into i: `axial`, or for a SymCompartment `distal`,
     * `sphere` or `cylinder`, as `link` below says) or -1.  Several children
     * of one parent joined by the same kind of link are connected in
     * increasing child index: that is the message order that
     * `HSolveUtils::adjacent`/`children` see (`hsolve/HSolveUtils.cpp:36-53`). */
    uint32_t n_compt;
    const int32_t* parent;
    const double* Ra;
    const double* Rm;
    const double* Cm;
    const double* Em;
    const double* initVm;
    const double* Vm;          /* value at setup (V_ before reinit) */
    const double* inject;      /* basal inject at setup              */

    /* Leakage channels (`HSolvePassive::initialize`, Thevenin sum). */
    uint32_t n_leak;
    const uint32_t* leak_compt;
    const double* leak_Ek;
    const double* leak_Gk;

    /* Prototype HHGate tables, shared by channels (`HSolveUtils::gates`
     * with getOriginals). */
    uint32_t n_gate;
    const HsGateTable* gate;

    /* HHChannels taken over by the solver (`readHHChannels`).  Channels of
     * one compartment are in message order = increasing channel index.   */
    uint32_t n_chan;
    const uint32_t* chan_compt;
    const double* chan_Gbar;
    const double* chan_Ek;
    const double* chan_Xpower;
    const double* chan_Ypower;
    const double* chan_Zpower;
    const int32_t* chan_xgate;       /* gate table index, or -1 */
    const int32_t* chan_ygate;
    const int32_t* chan_zgate;
    const int32_t* chan_instant;     /* bit 1 X, 2 Y, 4 Z          */
    const double* chan_modulation;
    const int32_t* chan_use_conc;    /* Z gate tabulated on Ca     */
    const double* chan_X;
    const double* chan_Y;
    const double* chan_Z;
    const int32_t* chan_ca_target;   /* pool fed by IkOut, or -1   */
    const int32_t* chan_ca_depend;   /* pool read by `concen`, or -1 */

    /* CaConc pools (`readCalcium`; B from shell volume,
     * `biophysics/CaConcBase.cpp:259-269`, is computed by the caller). */
    uint32_t n_pool;
    const uint32_t* pool_compt;
    const double* pool_Ca;
    const double* pool_CaBasal;
    const double* pool_tau;
    const double* pool_B;
    const double* pool_ceiling;
    const double* pool_floor;

    /* External HHChannel2D objects (tick 4; `biophysics/HHChannel2D.cpp:327-369`).
     * X gate only (Xpower > 0), looked up on (dep0, dep1) of `xindex`.  */
    uint32_t n_gate2d;
    const HsGate2DTable* gate2d;
    uint32_t n_chan2d;
    const uint32_t* c2d_compt;
    const double* c2d_Gbar;
    const double* c2d_Ek;
    const double* c2d_Xpower;
    const int32_t* c2d_xgate;        /* gate2d index */
    const int32_t* c2d_xindex;       /* HS_DEP_* */
    const int32_t* c2d_conc1_pool;   /* pool whose concOut feeds conc1, or -1 */
    const int32_t* c2d_conc2_pool;
    const int32_t* c2d_instant;
    const double* c2d_modulation;
    const double* c2d_X;             /* initial X (the `X` field set before reinit) */

    /* External SynChans (tick 4; `biophysics/SynChan.cpp:171-251`) with one
     * SimpleSynHandler each (tick 1; `synapse/SimpleSynHandler.cpp:86-119`). */
    uint32_t n_syn;
    const uint32_t* syn_compt;
    const double* syn_Gbar;
    const double* syn_Ek;
    const double* syn_tau1;
    const double* syn_tau2;
    const double* syn_modulation;
    /* Synaptic events already queued in each handler: event e arrives at
     * SynChan `ev_syn[e]` with time ev_time[e] (spike time + synapse delay)
     * and weight ev_weight[e].  Any order. */
    uint32_t n_event;
    const uint32_t* ev_syn;
    const double* ev_time;
    const double* ev_weight;

    /* SpikeGens driven by the solver (`readSynapses`, `SpikeGen::process`). */
    uint32_t n_spikegen;
    const uint32_t* sg_compt;
    const double* sg_threshold;
    const double* sg_refractT;
    const int32_t* sg_edge;

    /* Basal-inject schedule: before step stim_step[k] (0-based, counted from
     * reinit) the compartment's `inject` field is set to stim_value[k], as a
     * script does between `moose.start()` calls.  Sorted by step.        */
    uint32_t n_stim;
    const uint32_t* stim_compt;
    const uint32_t* stim_step;
    const double* stim_value;

    /* External calcium on tick 1, before the solver's tick 6: DifShells
     * (`biophysics/DifShell.cpp`), DifBuffers (`biophysics/DifBuffer.cpp`)
     * and MMPumps (`biophysics/MMPump.cpp`), listed in their tick-1 process
     * order, with HS_DIF_NPAR parameters each in `difpar` (layouts below).
     * Their messages, each (kind, src, dst) in creation order: a source's
     * sends reach its targets in that order, so the accumulations round as
     * in the reference.  The solver sends each HHChannel's Ik = (Ek - Vm) Gk
     * after its step (`HSolveActive::sendValues`,
     * `hsolve/HSolveActive.cpp:354-385`) to the shells its IkOut reaches,
     * and a shell's concentration reaches an HHChannel's `concen` as
     * `HSolve::addConc` does (`hsolve/HSolveInterface.cpp:254-259`). */
    uint32_t n_dif;
    const int32_t* dif_kind;       /* HS_DIF_* */
    const double* difpar;          /* n_dif x HS_DIF_NPAR */
    uint32_t n_dmsg;
    const int32_t* dmsg_kind;      /* HS_DMSG_* */
    const uint32_t* dmsg_src;      /* object (HHChannel for HS_DMSG_IK) */
    const uint32_t* dmsg_dst;      /* object (HHChannel for HS_DMSG_CONC_CHAN) */
    /* How each compartment hangs on its parent (n_compt entries, HS_LINK_*;
     * NULL: every link axial).  It places the parent and the children in
     * the order HSolveUtils::adjacent lists them -- axial targets, raxial,
     * distalOut, proximalOut, cylinderOut (hsolve/HSolveUtils.cpp:36-45) --
     * and the children in HSolveUtils::children's order (axial, distalOut,
     * cylinderOut), which set the Hines numbering and each junction's
     * operand order. */
    const int32_t* link;
} HsCellDesc;

#define HS_LINK_AXIAL    0   /* Compartment: parent axial -> child raxial      */
#define HS_LINK_DISTAL   1   /* SymCompartment: parent distal -> child proximal,
                                or parent sphere -> child proximalOnly        */
#define HS_LINK_CYLINDER 2   /* SymCompartment: parent cylinder -> child
                                proximalOnly (spines)                          */

/* tick-1 object kinds and their parameters (difpar, HS_DIF_NPAR per object) */
#define HS_DIF_SHELL   0   /* Ceq, D, valence, leak, shapeMode, length, diameter,
                              thickness, volume, outerArea, innerArea (the last
                              three used with shapeMode 3 only)            */
#define HS_DIF_BUFFER  1   /* bTot, kf, kb, D, shapeMode, length, diameter,
                              thickness, volume, outerArea, innerArea      */
#define HS_DIF_PUMP    2   /* Vmax, Kd                                     */
#define HS_DIF_NPAR   12
/* message kinds */
#define HS_DMSG_OUTER      0  /* outerDifSourceOut -> fluxFromOut (shell or buffer) */
#define HS_DMSG_INNER      1  /* innerDifSourceOut -> fluxFromIn                   */
#define HS_DMSG_CONC_CHAN  2  /* shell concentrationOut -> HHChannel concen         */
#define HS_DMSG_CONC_BUF   3  /* shell concentrationOut -> buffer concentration     */
#define HS_DMSG_REACTION   4  /* buffer reactionOut -> shell reaction               */
#define HS_DMSG_PUMP       5  /* pump PumpOut -> shell mmPump                        */
#define HS_DMSG_IK         6  /* HHChannel IkOut (sent by the solver) -> shell influx */

/* ------------------------------------------------------------------ */
/* Library */

/* Message for the last failing call on this thread. */
const char* hs_last_error(void);
/* Number of CUDA devices visible (0 when none); never fails. */
int hs_device_count(void);
/* Library build string (architecture and flags). */
const char* hs_build_info(void);

/* ------------------------------------------------------------------ */
/* Drop-in solver: one HSolve instance per cell.
 * Lifecycle mirrors `HSolve`: setPath/setup -> reinit -> process ...     */
typedef struct HsSolver HsSolver;

/* HSolve::setPath -> HSolve::setup (`hsolve/HSolve.cpp:286-334`):
 * `seed` is the compartment found under `target`; `dt` is the HSolve `dt`
 * field, used for the matrix, CmByDt and Ca factors.                    */
int hs_create(const HsCellDesc* cell, uint32_t seed, double dt, int precision,
              HsSolver** out);
int hs_destroy(HsSolver* s);

/* HSolve::reinit (`hsolve/HSolve.cpp:229-233`): `clock_dt` is the tick dt
 * used by gates, external objects and spike detection.                  */
int hs_reinit(HsSolver* s, double clock_dt);
/* nsteps calls of HSolve::process, with tick-1/4 external objects. */
int hs_process(HsSolver* s, uint32_t nsteps);
/* CTAs that step the solver's cell: 1 = one CTA; 2..8 = a thread-block
 * cluster whose CTAs share the channel and matrix-row work while one of them
 * eliminates (same arithmetic, bit-identical results); 0 (the default) =
 * by the cell's size (one CTA below 1,024 compartments, then one CTA per
 * 512 compartments, at most 8).  hs_get_cluster_ctas gives the number in
 * use.  No reference counterpart: a launch-shape choice. */
int hs_set_cluster_ctas(HsSolver* s, uint32_t ctas);
int hs_get_cluster_ctas(HsSolver* s, uint32_t* ctas);
/* hs_process(solvers[k], nsteps) for every k < n, in one launch per
 * cluster size: each solver is stepped by its own CTA (or cluster) with the
 * arithmetic hs_process uses, so the results are bit-identical.  For a Clock
 * tick that processes many HSolve objects (`scheduling/Clock.cpp:872-921`
 * calls each one's process in turn): one launch instead of one per solver,
 * all running at once.  The solvers keep their own streams; the launch is
 * ordered after the work already queued on each of them, and work queued on
 * any of them afterwards runs after it.  All solvers must be reinited
 * (HS_ESTATE), distinct and created on one device (HS_EINVAL); otherwise
 * nothing is launched. */
int hs_process_group(HsSolver* const* solvers, uint32_t n, uint32_t nsteps);
/* Wait for queued device work of this solver. */
int hs_sync(HsSolver* s);

/* Solver fields (`hsolve/HSolve.cpp:87-156`). */
int hs_set_ca_advance(HsSolver* s, int ca_advance);
int hs_get_ca_advance(HsSolver* s, int* out);
/* vMin,vMax,vDiv,caMin,caMax,caDiv after setup (recomputed from the gates,
 * `hsolve/HSolveActiveSetup.cpp:367-414`). */
int hs_get_table_grid(HsSolver* s, double* vmin, double* vmax, int* vdiv,
                      double* camin, double* camax, int* cadiv);
int hs_get_nsteps(HsSolver* s, uint64_t* out);

/* Zombie fields by (kind, field, model index).  Kinds and fields below. */
#define HS_KIND_COMPT   0
#define HS_KIND_CHAN    1
#define HS_KIND_POOL    2
#define HS_KIND_CHAN2D  3
#define HS_KIND_SYNCHAN 4

/* compartment fields (`hsolve/HSolveInterface.cpp:66-244`) */
#define HS_F_VM        0
#define HS_F_CM        1
#define HS_F_EM        2
#define HS_F_RM        3
#define HS_F_RA        4
#define HS_F_INITVM    5
#define HS_F_IM        6   /* read-only */
#define HS_F_INJECT    7
/* channel fields (`hsolve/HSolveInterface.cpp:262-451`) */
#define HS_F_GBAR     10
#define HS_F_EK       11
#define HS_F_GK       12
#define HS_F_IK       13   /* read-only */
#define HS_F_X        14
#define HS_F_Y        15
#define HS_F_Z        16
#define HS_F_INSTANT  17
#define HS_F_MODULATION 18
#define HS_F_XPOWER   19
#define HS_F_YPOWER   20
#define HS_F_ZPOWER   21
/* pool fields (`hsolve/HSolveInterface.cpp:453-533`) */
#define HS_F_CA       30
#define HS_F_CABASAL  31
#define HS_F_CEILING  32
#define HS_F_FLOOR    33
#define HS_F_TAU      34   /* write-only pair with B: set both via hs_set_tau_b */
#define HS_F_B        35

/* Between process calls, reads are served from a host mirror of the
 * solver's device memory (refreshed page by page after each process), and
 * writes are queued and applied before the next process, reinit or bulk
 * read; a read always sees the writes made before it. */
int hs_get_field(HsSolver* s, int kind, int field, uint32_t index, double* out);
int hs_set_field(HsSolver* s, int kind, int field, uint32_t index, double value);
int hs_set_tau_b(HsSolver* s, uint32_t pool, double tau, double B);

/* Message destinations into the solver, applied at the next step only
 * (`HSolve::addInject`, `addGkEk`, `addConc`, `iCa`). */
int hs_add_inject(HsSolver* s, uint32_t compt, double value);
int hs_add_gkek(HsSolver* s, uint32_t compt, double Gk, double Ek);
int hs_add_conc(HsSolver* s, uint32_t chan, double conc);
int hs_add_ica(HsSolver* s, uint32_t pool, double ica);

/* Synaptic events at run time: event e is queued in the SimpleSynHandler of
 * SynChan `syn[e]` with delivery time time[e] and weight weight[e]
 * (`SimpleSynHandler::addSpike`, `synapse/SimpleSynHandler.cpp:86-90`; the
 * caller adds the synapse delay, as `Synapse::addSpike` does at
 * `synapse/Synapse.cpp:104-113`).  An event is delivered at the first step
 * whose clock time is >= its time, as weight/dt into the SynChan's
 * activation (`SimpleSynHandler::vProcess`, lines 98-113), including events
 * whose time has already passed.  Events with equal times on one SynChan
 * are summed in the order they were pushed, after the description's.
 * reinit drops every queued runtime event (`SimpleSynHandler::vReinit`).
 * Times must not be NaN.  The events reach the device at the next
 * hs_process. */
int hs_push_events(HsSolver* s, const uint32_t* syn, const double* time,
                   const double* weight, uint32_t n);

/* Bulk reads in model order (n = n_compt / n_pool). */
int hs_read_vm(HsSolver* s, double* out, uint32_t n);
int hs_read_ca(HsSolver* s, double* out, uint32_t n);

/* Tick-1 external calcium objects in description order: C of each
 * DifShell, bFree of each DifBuffer, 0 for an MMPump (n = n_dif). */
int hs_read_dif(HsSolver* s, double* out, uint32_t n);

/* Trace recording: every `stride` steps, Vm of the listed compartments is
 * appended to a device buffer (a Table on tick 8 reading `HSolve::getVm`). */
int hs_record(HsSolver* s, const uint32_t* compts, uint32_t n, uint32_t stride,
              uint32_t capacity_samples);
/* The values the solver sends each step to objects it does not own
 * (`HSolveActive::sendValues`, hsolve/HSolveActive.cpp:354-385), recorded
 * on the device every `stride` steps: entry r is the Vm of compartment
 * index[r] (kind HS_KIND_COMPT, field HS_F_VM: VmOut), the Ik = (Ek - Vm) Gk
 * (HS_KIND_CHAN, HS_F_IK: IkOut) or Gk (HS_F_GK) of an HHChannel, or the Ca
 * of a pool (HS_KIND_POOL, HS_F_CA: concOut).  Replaces the recording of
 * hs_record (which records Vm only); read with hs_read_trace. */
int hs_record_values(HsSolver* s, const int* kind, const int* field, const uint32_t* index, uint32_t n,
                     uint32_t stride, uint32_t capacity);
int hs_read_trace(HsSolver* s, double* out, uint32_t capacity, uint32_t* n_samples);

/* Spikes from the SpikeGens: (spikegen model index, time) pairs. */
int hs_read_spikes(HsSolver* s, uint32_t* gen, double* time, uint32_t capacity,
                   uint32_t* n);

/* ------------------------------------------------------------------ */
/* Batched solver: many cells packed by size into one persistent kernel.
 * No counterpart in the reference (it runs one serial HSolve per cell).  */
typedef struct HsBatch HsBatch;

/* Launch shape of the batched kernel (0 keeps the current value).
 * FP64: one wave of ctas_per_sm x SM-count CTAs (fewer per SM if the
 * kernel's registers do not fit that many); a warp steps its cells one after
 * the other, and the cells too large to share a warp's load with others are
 * stepped by a whole CTA each.  Mixed: one CTA steps a forest of cells at a time; a forest
 * holds its elimination arrays in the CTA's shared memory (30 B per node),
 * so ctas_per_sm and forest_nodes set the forest size.  Changing either (or
 * max_ctas) on a mixed batch renumbers its nodes: its state, recording and
 * inject targets start over and hs_batch_reinit must follow. */
typedef struct HsBatchTuning {
    uint32_t threads_per_cta;   /* multiple of 32; FP64 <= 256 (default 128),
                                   mixed <= 1024 (default 1024) */
    uint32_t ctas_per_sm;       /* CTAs per SM (default 4 FP64, 1 mixed) */
    uint32_t steps_per_launch;  /* dt steps per kernel launch (default 100) */
    uint32_t use_graph;         /* capture a process() call as a CUDA graph */
    uint32_t forest_nodes;      /* mixed: most nodes per shared-memory forest
                                   (0: as many as shared memory holds) */
    uint32_t max_ctas;          /* mixed: pack the cells into at most this many
                                   CTAs (0: ctas_per_sm x SM count); fewer,
                                   fuller forests leave SMs to other batches */
    uint32_t elim_warps;        /* mixed: warps of a CTA that eliminate while the
                                   others assemble (default 4; 0 keeps the
                                   current value, 0xFFFFFFFF turns the split off) */
    uint32_t wait_rounds;       /* mixed: most sleep rounds (~128 ns each) an
                                   eliminator waits for one level's assembly
                                   before it gives up; after that the launch
                                   waits no more, finishes its steps and
                                   hs_batch_sync returns HS_ETIMEOUT until the
                                   next reinit (default 2^24, about 2 s; 0 keeps
                                   the current value) */
    uint32_t cluster_ctas;      /* mixed: CTAs (SMs) that step each group of
                                   forests together, as one thread-block
                                   cluster (0 or 1: one CTA per group, the
                                   throughput layout; 2..8: a large cell
                                   assembled by several SMs, for latency).
                                   With 2 or more every forest is eliminated
                                   in global memory and may have at most 255
                                   levels (else HS_ENOTSUP); changing it
                                   re-lays the batch out. */
} HsBatchTuning;

int hs_batch_create(const HsCellDesc* cells, const uint32_t* seeds,
                    uint32_t n_cells, double dt, int precision,
                    const HsBatchTuning* tuning, HsBatch** out);
int hs_batch_destroy(HsBatch* b);
/* Re-pack the cells for a new launch shape (the autotuner's knob). */
int hs_batch_tune(HsBatch* b, const HsBatchTuning* tuning);
int hs_batch_reinit(HsBatch* b, double clock_dt);
int hs_batch_process(HsBatch* b, uint32_t nsteps);
int hs_batch_sync(HsBatch* b);
/* *idle = 1 when all queued work of the batch has finished, else 0; does
 * not wait. */
int hs_batch_idle(HsBatch* b, int* idle);
/* Vm of every compartment of cell `cell` in model order. */
int hs_batch_read_vm(HsBatch* b, uint32_t cell, double* out, uint32_t n);
int hs_batch_read_ca(HsBatch* b, uint32_t cell, double* out, uint32_t n);
/* Vm (field HS_F_VM) or Ca (HS_F_CA) of every compartment (pool) of every
 * cell, cell after cell, each cell in model order: n = the batch's total
 * compartment (pool) count.  One gather on the device and one copy,
 * whatever the number of cells: the chunk-boundary form of the solver's
 * outgoing VmOut/concOut values (`HSolveActive::sendValues`,
 * hsolve/HSolveActive.cpp:342-385) for a whole population. */
int hs_batch_read_all(HsBatch* b, int field, double* out, uint64_t n);
int hs_batch_record(HsBatch* b, const uint32_t* cell, const uint32_t* compt,
                    uint32_t n, uint32_t stride, uint32_t capacity_samples);
int hs_batch_read_trace(HsBatch* b, double* out, uint32_t capacity,
                        uint32_t* n_samples);
/* Samples [first, first+count) of the recording (rows of all recorded
 * columns), e.g. the samples of the last process() call. */
int hs_batch_read_trace_window(HsBatch* b, uint32_t first, uint32_t count,
                               double* out);
/* Writing the `inject` field of many compartments between process() calls
 * (ZombieCompartment inject -> HSolve::setInject): register the targets
 * once, then copy one value per target from host memory (pinned memory makes
 * the copy asynchronous); the values apply from the next step. */
int hs_batch_inject_targets(HsBatch* b, const uint32_t* cell, const uint32_t* compt,
                            uint32_t n);
int hs_batch_set_inject(HsBatch* b, const double* values, uint32_t n);
/* The modulation field of channels of a batch between process() calls, as
 * a chem->elec Adaptor (signeur/Adaptor.cpp) sets it each step: kind
 * HS_KIND_CHAN = HHChannel k of cells[k] (HSolve::setHHmodulation,
 * hsolve/HSolveInterface.cpp:445-451: a value <= 0 keeps the old one),
 * HS_KIND_CHAN2D / HS_KIND_SYNCHAN = that HHChannel2D / SynChan
 * (ChanCommon::vSetModulation, biophysics/ChanCommon.cpp:46-49).  Indices
 * are the cell description's; the values apply from the next step and
 * persist across reinit and repacking.  Returns after the writes are done. */
int hs_batch_set_modulation(HsBatch* b, int kind, const uint32_t* cells, const uint32_t* index,
                            const double* values, uint32_t n);
/* Synaptic events queued at run time on batched cells: hs_push_events for
 * many cells in one call (SimpleSynHandler::addSpike,
 * synapse/SimpleSynHandler.cpp:86-90).  Event e reaches SynChan syn[e] (the
 * cell's description index) of cell cell[e] at time time[e] (spike time +
 * synapse delay) with weight weight[e]; it is delivered at the first step
 * whose clock time is >= its time, including times already passed.  Events
 * with equal times on one SynChan are summed in push order, after the ones
 * already queued.  The pushes reach the device at the next
 * hs_batch_process; hs_batch_reinit and a re-layout by hs_batch_tune drop
 * every queued runtime event.  Both precisions; in the mixed batch the
 * delivery step is taken at the clock dt of the last reinit.  Validates
 * every event before queuing any (HS_EINVAL: cell or SynChan out of range,
 * NaN time). */
int hs_batch_push_events(HsBatch* b, const uint32_t* cell, const uint32_t* syn, const double* time,
                         const double* weight, uint32_t n);
/* The inject of compartment compt[k] of cell cell[k] becomes values[k], for
 * k < n, without allocating any memory: the writes go through a fixed
 * host staging array and a fixed device scratch array of 32768 entries
 * (larger n: HS_ECAPACITY).  For callers that must not allocate between
 * process() calls, such as a loop driving other batches on the same GPU
 * (cudaMalloc/cudaFree would wait for the whole device).  The first call on
 * a device looks up the scratch address and should come before any stream
 * capture on it; calls share the storage, are serialised by a lock and
 * return after the writes are done.  Same targets and rules as
 * hs_batch_inject_targets + hs_batch_set_inject.  Name each (cell, compt)
 * pair at most once per call: a pair named twice gets one of its values,
 * which one is not defined.  The scratch address is looked up once per
 * device and kept, which assumes the device's primary context is not reset
 * (cudaDeviceReset) while the library is loaded.  No counterpart in the
 * reference. */
int hs_batch_set_inject_at(HsBatch* b, const uint32_t* cell, const uint32_t* compt,
                           const double* values, uint32_t n);
int hs_batch_read_spikes(HsBatch* b, uint32_t* cell, uint32_t* gen,
                         double* time, uint32_t capacity, uint32_t* n);
/* Serving support (mixed batch).  Cell c advances only while its step count
 * is below stop[c] (UINT64_MAX: no limit; set before or between process()
 * calls); a stopped cell keeps its final state, trace and spikes.  n equals
 * the number of cells.  No counterpart in the reference, which steps every
 * compartment on every tick. */
int hs_batch_set_stop_steps(HsBatch* b, const uint64_t* stop, uint32_t n);
/* dt steps each cell has advanced (at most its stop step). */
int hs_batch_read_steps(HsBatch* b, uint64_t* out, uint32_t n);
/* Spikes recorded so far by each cell. */
int hs_batch_read_spike_counts(HsBatch* b, uint32_t* out, uint32_t n);
/* One round trip for a serving loop: trace samples [first, first+count)
 * (as hs_batch_read_trace_window), each cell's step count and spike count
 * (n_cells entries each); any output may be null. */
int hs_batch_poll(HsBatch* b, uint32_t first, uint32_t count, double* trace, uint64_t* steps,
                  uint32_t* spike_counts);
/* Device memory held by the batch, in bytes. */
int hs_batch_device_bytes(HsBatch* b, uint64_t* out);
/* Spikes of one cell from its `first`-th on; *n = the cell's total count.
 * Returns HS_ECAPACITY if the per-cell spike buffer overflowed. */
int hs_batch_read_cell_spikes(HsBatch* b, uint32_t cell, uint32_t first, uint32_t* gen,
                              double* time, uint32_t capacity, uint32_t* n);
/* The CUDA stream (a cudaStream_t) the batch runs on, for event timing. */
int hs_batch_stream(HsBatch* b, void** stream);
/* Statistics of the packing: compartments, cells, CTAs, launches/step. */
int hs_batch_info(HsBatch* b, uint64_t* n_compt, uint32_t* n_ctas,
                  uint32_t* threads_per_cta, uint32_t* steps_per_launch);
/* Mixed batch: how many elimination forests the packing made and how many
 * of them are eliminated in shared memory (the others in global memory);
 * 0 and 0 for an FP64 batch. */
int hs_batch_forests(HsBatch* b, uint32_t* n_forests, uint32_t* n_shared);
/* Average duration (ms) of the stepping kernel launches timed with CUDA
 * events on the batch's stream since the last call, and their count. */
int hs_batch_kernel_time(HsBatch* b, double* avg_ms, uint32_t* launches);

#ifdef __cplusplus
}
#endif
#endif /* MOOSE_GB300_H */
