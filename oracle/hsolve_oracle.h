/*
 * hsolve_oracle.h -- CPU restatement of MOOSE HSolve (test infrastructure).
 *
 * This is the ORACLE: a plain-C, single-threaded restatement of the
 * reference's HSolve setup and per-step arithmetic, in the reference's own
 * operation order.  It exists only to check the GPU product and to time a
 * CPU baseline.  Nothing in the product links or calls it; only tests/,
 * __graft_entry__.smoke() and bench.py's CPU legs do.
 *
 * Reference files restated (paths inside the reference project):
 *   hsolve/HSolvePassive.cpp   walkTree 45-98, initialize 100-165,
 *                              storeTree 167-205, updateMatrix 211-244,
 *                              forwardEliminate 246-323, backwardSubstitute 325-401
 *   hsolve/HinesMatrix.cpp     setup 25-51, makeJunctions 84-130,
 *                              makeMatrix 133-223, makeOperands 226-365, getA 509-552
 *   hsolve/HSolveActive.cpp    step 45-66, calculateChannelCurrents 68-83,
 *                              updateMatrix 85-151, advanceCalcium 153-216,
 *                              advanceChannels 218-332
 *   hsolve/HSolveActiveSetup.cpp  reinit 43-160, readHHChannels 162-235,
 *                              readGates 237-250, readCalcium 252-337,
 *                              createLookupTables 339-526
 *   hsolve/RateLookup.cpp      LookupTable 15-103
 *   hsolve/HSolveStruct.cpp    ChannelStruct 15-65, CaConcStruct 108-155
 *   hsolve/HSolveUtils.cpp     rates 215-252 (resampling via HHGate::lookupBoth,
 *                              biophysics/HHGate.cpp:258-283)
 *   biophysics/HHChannel2D.cpp 327-369, biophysics/HHChannelBase.cpp 268-274, 330-348
 *   builtins/Interpol2D.cpp    508-592
 *   biophysics/SynChan.cpp     171-251, synapse/SimpleSynHandler.cpp 86-119
 *   biophysics/SpikeGen.cpp    202-222
 *   scheduling/Clock.cpp       702-774 (currTime = dt * endStep; tick order)
 */
#ifndef HSOLVE_ORACLE_H
#define HSOLVE_ORACLE_H

#include <stdint.h>
#include "../include/moose_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct OrcCell OrcCell;

/* HSolve::setup on a cell description; returns NULL and fills err on error. */
OrcCell* orc_create(const HsCellDesc* d, uint32_t seed, double dt,
                    char* err, uint32_t errlen);
void orc_destroy(OrcCell* c);
void orc_set_ca_advance(OrcCell* c, int ca_advance);
/* Conditioning probe for accuracy analysis, off by default: gate increments
   computed in FP32 and accumulated in FP64 (the gating precision of a
   mixed-precision solver) instead of the reference's FP64 step. */
void orc_set_f32_gate_increments(OrcCell* c, int on);
/* Tick-1 external calcium objects: C of each DifShell, bFree of each
   DifBuffer, 0 for an MMPump (n_dif values). */
void orc_read_dif(const OrcCell* c, double* out);
/* HSolve::reinit with the clock dt (also reinit of tick-1/4 objects). */
void orc_reinit(OrcCell* c, double clock_dt);
/* nsteps clock steps: ticks 0 (stimulus), 1, 4, 6 (HSolve), spikes. */
void orc_step(OrcCell* c, uint32_t nsteps);

uint32_t orc_n_compt(const OrcCell* c);
uint32_t orc_n_pool(const OrcCell* c);
uint32_t orc_n_state(const OrcCell* c);
/* Hines index of a model compartment. */
uint32_t orc_hines_index(const OrcCell* c, uint32_t model_compt);
/* Model index of the compartment at a Hines index. */
uint32_t orc_model_index(const OrcCell* c, uint32_t hines);
/* Vm of all compartments in model order. */
void orc_read_vm(const OrcCell* c, double* out);
/* Ca of all pools, in model (descriptor) pool order; pools not taken by the
 * solver report NaN. */
void orc_read_ca(const OrcCell* c, double* out);
/* Gate states in solver order (state_ vector). */
void orc_read_state(const OrcCell* c, double* out);
/* Spikes: returns the count; copies up to cap (model spikegen index, time). */
uint32_t orc_read_spikes(const OrcCell* c, uint32_t* gen, double* t, uint32_t cap);
/* Table grid after setup (vMin_, vMax_, vDiv_, caMin_, caMax_, caDiv_). */
void orc_table_grid(const OrcCell* c, double* g6);
/* Field access mirroring HSolveInterface (model indices). */
int orc_get_field(const OrcCell* c, int kind, int field, uint32_t index, double* out);
int orc_set_field(OrcCell* c, int kind, int field, uint32_t index, double value);
/* Message destinations (HSolve::addInject, addGkEk, addConc, iCa), model
 * indices; 0 or HS_EINVAL. */
int orc_add_inject(OrcCell* c, uint32_t compt, double value);
int orc_add_gkek(OrcCell* c, uint32_t compt, double Gk, double Ek);
int orc_add_conc(OrcCell* c, uint32_t chan, double conc);
int orc_add_ica(OrcCell* c, uint32_t pool, double ica);
/* Synaptic event queued at run time (SimpleSynHandler::addSpike): delivered
 * at the first step whose clock time is >= time, as weight/dt; dropped by
 * reinit.  0, or HS_EINVAL for a bad index or a NaN time. */
int orc_push_event(OrcCell* c, uint32_t syn, double time, double weight);

/* Passive known-answer interface (HinesMatrix/HSolvePassive unit tests):
 * tree given directly in Hines order as child lists (CSR). */
OrcCell* orc_passive_create(uint32_t n, const uint32_t* child_off,
                            const uint32_t* child_idx, const double* Ra,
                            const double* Rm, const double* Cm,
                            const double* Em, const double* V, double dt);
void orc_passive_update(OrcCell* c);     /* HSolvePassive::updateMatrix */
void orc_forward(OrcCell* c);            /* forwardEliminate */
void orc_backward(OrcCell* c);           /* backwardSubstitute */
double orc_getA(const OrcCell* c, uint32_t row, uint32_t col);
double orc_getB(const OrcCell* c, uint32_t row);
double orc_getVMid(const OrcCell* c, uint32_t row);
double orc_getV(const OrcCell* c, uint32_t row);

#ifdef __cplusplus
}
#endif
#endif
