// hsolve_gpu.hpp -- the HSolve class interface in C++, on the C ABI of
// libmoose_gb300 (include/moose_gb300.h).  Header only.
//
// It mirrors the public interface of the reference's HSolve
// (hsolve/HSolve.h:20-179, hsolve/HSolve.cpp, hsolve/HSolveInterface.cpp):
// the solver fields dt, caAdvance, vDiv/vMin/vMax, caDiv/caMin/caMax;
// setup from a seed compartment (HSolve::setPath -> setup); reinit and
// process; the zombie fields of compartments, HHChannels and CaConcs; and
// the message destinations addInject, addGkEk, addConc, iCa and the
// synaptic events of SimpleSynHandler::addSpike.  A MOOSE
// build keeps its HSolve Cinfo and forwards to this class (or to the C ABI
// directly); other C++ hosts use it as the solver object.
//
// Where the reference takes an Id, this class takes the model index of the
// object in the cell description (HsCellDesc): compartment, HHChannel or
// CaConc number.  Errors: like HSolve::setPath, setTarget prints the reason
// to std::cerr and leaves the solver unset (returns false); every other
// call that the C ABI rejects (no solver, index out of range, device error)
// throws moose_gb300::Error with the status code and message -- the
// reference asserts on an unknown Id instead (hsolve/HSolveInterface.cpp:33).
#pragma once

#include <cmath>
#include <cstdint>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "moose_gb300.h"

namespace moose_gb300 {

class Error : public std::runtime_error {
public:
    Error(int code, const std::string& msg) : std::runtime_error(msg), code_(code) {}
    int code() const { return code_; }

private:
    int code_;
};

inline void check(int rc) {
    if (rc != HS_OK) throw Error(rc, hs_last_error());
}

class HSolve {
public:
    HSolve() = default;
    ~HSolve() {
        if (s_) hs_destroy(s_);
    }
    HSolve(const HSolve&) = delete;
    HSolve& operator=(const HSolve&) = delete;

    // ---- solver fields (hsolve/HSolve.cpp:87-156, 409-499)
    void setDt(double dt) {
        if (dt < 0.0) {
            std::cerr << "Error: HSolve: 'dt' must be positive.\n";
            return;
        }
        dt_ = dt;
    }
    double getDt() const { return dt_; }
    void setCaAdvance(int caAdvance) {
        if (caAdvance != 0 && caAdvance != 1) {
            std::cerr << "Error: HSolve: caAdvance should be either 0 or 1.\n";
            return;
        }
        caAdvance_ = caAdvance;
        if (s_) check(hs_set_ca_advance(s_, caAdvance));
    }
    int getCaAdvance() const { return caAdvance_; }
    // The table grid is recomputed from the gates at setup
    // (hsolve/HSolveActiveSetup.cpp:367-414): the values set here are
    // reported until then and ignored by the solver, as in the reference
    // (whose values before setup are unset; the defaults below are the
    // Python mirror's).
    void setVDiv(int v) { vDiv_ = v; }
    void setVMin(double v) { vMin_ = v; }
    void setVMax(double v) { vMax_ = v; }
    void setCaDiv(int v) { caDiv_ = v; }
    void setCaMin(double v) { caMin_ = v; }
    void setCaMax(double v) { caMax_ = v; }
    int getVDiv() const { return s_ ? grid().vdiv : vDiv_; }
    double getVMin() const { return s_ ? grid().vmin : vMin_; }
    double getVMax() const { return s_ ? grid().vmax : vMax_; }
    int getCaDiv() const { return s_ ? grid().cadiv : caDiv_; }
    double getCaMin() const { return s_ ? grid().camin : caMin_; }
    double getCaMax() const { return s_ ? grid().camax : caMax_; }

    // ---- setup (HSolve::setPath -> setup, hsolve/HSolve.cpp:286-334): the
    // cell description and the compartment the tree walk starts from.  The
    // description's arrays must stay valid while the solver is created.
    bool setTarget(const HsCellDesc& cell, uint32_t seed) {
        if (dt_ == 0.0) {
            std::cerr << "Error: HSolve::setPath(): Must set 'dt' first.\n";
            return false;
        }
        if (s_) {
            hs_destroy(s_);
            s_ = nullptr;
        }
        HsSolver* s = nullptr;
        const int rc = hs_create(&cell, seed, dt_, HS_PREC_FP64, &s);
        if (rc != HS_OK) {
            std::cerr << "Error: HSolve::setup: " << hs_last_error() << "\n";
            return false;
        }
        s_ = s;
        seed_ = seed;
        check(hs_set_ca_advance(s_, caAdvance_));
        return true;
    }
    bool ready() const { return s_ != nullptr; }
    uint32_t getSeed() const { return seed_; }

    // ---- proc (hsolve/HSolve.cpp:221-233)
    void reinit(double clockDt) {
        check(hs_reinit(handle(), clockDt));
        dt_ = clockDt;
    }
    void process(uint32_t nsteps = 1) { check(hs_process(handle(), nsteps)); }
    void sync() { check(hs_sync(handle())); }
    // The process of every HSolve of a clock tick in one launch
    // (hs_process_group; the Clock calls them in turn,
    // scheduling/Clock.cpp:872-921), bit-identical to each process().
    static void processGroup(const std::vector<HSolve*>& tick, uint32_t nsteps = 1) {
        std::vector<HsSolver*> s;
        s.reserve(tick.size());
        for (HSolve* h : tick) s.push_back(h->handle());
        check(hs_process_group(s.data(), (uint32_t)s.size(), nsteps));
    }
    // CTAs stepping this cell: 0 = by its size, 1 = one, 2..8 = a cluster.
    void setClusterCtas(uint32_t n) { check(hs_set_cluster_ctas(handle(), n)); }
    uint32_t getClusterCtas() const {
        uint32_t n = 0;
        check(hs_get_cluster_ctas(handle(), &n));
        return n;
    }
    uint64_t steps() const {
        uint64_t n = 0;
        check(hs_get_nsteps(handle(), &n));
        return n;
    }

    // ---- compartment fields (hsolve/HSolveInterface.cpp:45-224)
    double getVm(uint32_t c) const { return get(HS_KIND_COMPT, HS_F_VM, c); }
    void setVm(uint32_t c, double v) { set(HS_KIND_COMPT, HS_F_VM, c, v); }
    double getInitVm(uint32_t c) const { return get(HS_KIND_COMPT, HS_F_INITVM, c); }
    void setInitVm(uint32_t c, double v) { set(HS_KIND_COMPT, HS_F_INITVM, c, v); }
    double getCm(uint32_t c) const { return get(HS_KIND_COMPT, HS_F_CM, c); }
    void setCm(uint32_t c, double v) { set(HS_KIND_COMPT, HS_F_CM, c, v); }
    double getEm(uint32_t c) const { return get(HS_KIND_COMPT, HS_F_EM, c); }
    void setEm(uint32_t c, double v) { set(HS_KIND_COMPT, HS_F_EM, c, v); }
    double getRm(uint32_t c) const { return get(HS_KIND_COMPT, HS_F_RM, c); }
    void setRm(uint32_t c, double v) { set(HS_KIND_COMPT, HS_F_RM, c, v); }
    double getRa(uint32_t c) const { return get(HS_KIND_COMPT, HS_F_RA, c); }
    void setRa(uint32_t c, double v) { set(HS_KIND_COMPT, HS_F_RA, c, v); }
    double getIm(uint32_t c) const { return get(HS_KIND_COMPT, HS_F_IM, c); }
    double getInject(uint32_t c) const { return get(HS_KIND_COMPT, HS_F_INJECT, c); }
    void setInject(uint32_t c, double v) { set(HS_KIND_COMPT, HS_F_INJECT, c, v); }

    // ---- HHChannel fields (hsolve/HSolveInterface.cpp:262-451)
    double getHHChannelGbar(uint32_t k) const { return get(HS_KIND_CHAN, HS_F_GBAR, k); }
    void setHHChannelGbar(uint32_t k, double v) { set(HS_KIND_CHAN, HS_F_GBAR, k, v); }
    double getEk(uint32_t k) const { return get(HS_KIND_CHAN, HS_F_EK, k); }
    void setEk(uint32_t k, double v) { set(HS_KIND_CHAN, HS_F_EK, k, v); }
    double getGk(uint32_t k) const { return get(HS_KIND_CHAN, HS_F_GK, k); }
    void setGk(uint32_t k, double v) { set(HS_KIND_CHAN, HS_F_GK, k, v); }
    double getIk(uint32_t k) const { return get(HS_KIND_CHAN, HS_F_IK, k); }
    double getX(uint32_t k) const { return get(HS_KIND_CHAN, HS_F_X, k); }
    void setX(uint32_t k, double v) { set(HS_KIND_CHAN, HS_F_X, k, v); }
    double getY(uint32_t k) const { return get(HS_KIND_CHAN, HS_F_Y, k); }
    void setY(uint32_t k, double v) { set(HS_KIND_CHAN, HS_F_Y, k, v); }
    double getZ(uint32_t k) const { return get(HS_KIND_CHAN, HS_F_Z, k); }
    void setZ(uint32_t k, double v) { set(HS_KIND_CHAN, HS_F_Z, k, v); }
    int getInstant(uint32_t k) const { return (int)get(HS_KIND_CHAN, HS_F_INSTANT, k); }
    void setInstant(uint32_t k, int v) { set(HS_KIND_CHAN, HS_F_INSTANT, k, (double)v); }
    void setPowers(uint32_t k, double x, double y, double z) {
        set(HS_KIND_CHAN, HS_F_XPOWER, k, x);
        set(HS_KIND_CHAN, HS_F_YPOWER, k, y);
        set(HS_KIND_CHAN, HS_F_ZPOWER, k, z);
    }
    // a value <= 0 keeps the old modulation (HSolve::setHHmodulation)
    void setHHmodulation(uint32_t k, double v) { set(HS_KIND_CHAN, HS_F_MODULATION, k, v); }

    // ---- CaConc fields (hsolve/HSolveInterface.cpp:453-533)
    double getCa(uint32_t p) const { return get(HS_KIND_POOL, HS_F_CA, p); }
    void setCa(uint32_t p, double v) { set(HS_KIND_POOL, HS_F_CA, p, v); }
    double getCaBasal(uint32_t p) const { return get(HS_KIND_POOL, HS_F_CABASAL, p); }
    void setCaBasal(uint32_t p, double v) { set(HS_KIND_POOL, HS_F_CABASAL, p, v); }
    void setTauB(uint32_t p, double tau, double B) { check(hs_set_tau_b(handle(), p, tau, B)); }
    double getCaCeiling(uint32_t p) const { return get(HS_KIND_POOL, HS_F_CEILING, p); }
    void setCaCeiling(uint32_t p, double v) { set(HS_KIND_POOL, HS_F_CEILING, p, v); }
    double getCaFloor(uint32_t p) const { return get(HS_KIND_POOL, HS_F_FLOOR, p); }
    void setCaFloor(uint32_t p, double v) { set(HS_KIND_POOL, HS_F_FLOOR, p, v); }

    // ---- message destinations (HSolve::addInject, addGkEk, addConc, iCa):
    // they apply to the next step only
    void addInject(uint32_t c, double v) { check(hs_add_inject(handle(), c, v)); }
    void addGkEk(uint32_t c, double Gk, double Ek) { check(hs_add_gkek(handle(), c, Gk, Ek)); }
    void addConc(uint32_t k, double conc) { check(hs_add_conc(handle(), k, conc)); }
    void iCa(uint32_t p, double ica) { check(hs_add_ica(handle(), p, ica)); }
    // SimpleSynHandler::addSpike for SynChan k's handler (time includes the
    // synapse delay, as Synapse::addSpike adds it); delivered from the next
    // process() on, dropped by reinit()
    void addSpike(uint32_t k, double time, double weight) {
        check(hs_push_events(handle(), &k, &time, &weight, 1));
    }

    // ---- bulk reads in model order (a Table per compartment would need
    // a device read per field access)
    std::vector<double> vm(uint32_t nCompt) const {
        std::vector<double> out(nCompt);
        check(hs_read_vm(handle(), out.data(), nCompt));
        return out;
    }
    std::vector<double> ca(uint32_t nPool) const {
        std::vector<double> out(nPool);
        if (nPool) check(hs_read_ca(handle(), out.data(), nPool));
        return out;
    }
    // SpikeGen spikes since reinit: (spikegen index, time) pairs
    void spikes(std::vector<uint32_t>& gen, std::vector<double>& t) const {
        uint32_t n = 0;
        check(hs_read_spikes(handle(), nullptr, nullptr, 0, &n));
        gen.resize(n);
        t.resize(n);
        if (n) check(hs_read_spikes(handle(), gen.data(), t.data(), n, &n));
    }

    HsSolver* handle() const {
        if (!s_) throw Error(HS_EINVAL, "HSolve: no solver (setTarget has not succeeded)");
        return s_;
    }

private:
    struct Grid {
        double vmin, vmax, camin, camax;
        int vdiv, cadiv;
    };
    Grid grid() const {
        Grid g{};
        check(hs_get_table_grid(s_, &g.vmin, &g.vmax, &g.vdiv, &g.camin, &g.camax, &g.cadiv));
        return g;
    }
    double get(int kind, int field, uint32_t i) const {
        double v = NAN;
        check(hs_get_field(handle(), kind, field, i, &v));
        return v;
    }
    void set(int kind, int field, uint32_t i, double v) { check(hs_set_field(handle(), kind, field, i, v)); }

    HsSolver* s_ = nullptr;
    double dt_ = 50e-6;          // HSolve's default dt (hsolve/HSolve.cpp:197-200)
    int caAdvance_ = 1;          // hsolve/HSolveActive.cpp:33-40
    uint32_t seed_ = 0;
    int vDiv_ = 3000, caDiv_ = 3000;
    double vMin_ = -0.1, vMax_ = 0.05, caMin_ = 0.0, caMax_ = 1.0;
};

}  // namespace moose_gb300
