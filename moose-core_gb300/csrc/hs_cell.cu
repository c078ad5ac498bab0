// hs_cell.cu -- upload of a CellPlan into a device arena (see hs_cell.h).
#include <cstring>

#include "hs_cell.h"

namespace hsg {

namespace {

struct Uploader {
    Arena& a;
    cudaStream_t st;
    cudaError_t err = cudaSuccess;
    template <class T>
    T* put(const std::vector<T>& v, size_t n = 0) {
        size_t cnt = n ? n : v.size();
        T* p = a.take<T>(cnt ? cnt : 1);
        if (a.base && !v.empty() && err == cudaSuccess)
            err = cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st);
        return p;
    }
    template <class T>
    T* zeros(size_t n) {
        return a.take<T>(n ? n : 1);    // the arena is memset to 0 before upload
    }
};

}  // namespace

cudaError_t layoutCell(const CellPlan& P, Arena& a, DevCell& c, uint32_t spikeCap,
                       cudaStream_t st, const CellShared* sh) {
    Uploader u{a, st};
    const uint32_t N = P.N, H = P.H;
    std::memset(&c, 0, sizeof(c));
    c.N = N; c.H = H; c.C = P.C; c.G = P.G; c.P = P.P; c.K2 = P.K2; c.S = P.S; c.SG = P.SG;
    c.nStim = (uint32_t)P.stimStep.size();
    c.fLevels = (uint32_t)P.fLevelPtr.size() - 1;
    c.bLevels = (uint32_t)P.bLevelPtr.size() - 1;
    c.caAdvance = 1;
    c.dt = P.dtSetup;
    c.V = u.put(P.V0);
    c.initVm = sh ? sh->initVm : u.put(P.initVm);
    c.synConst = sh ? sh->synConst : u.zeros<double>(5 * (size_t)P.S);
    c.c2dX0 = u.put(P.c2dX0);
    c.VMid = u.zeros<double>(N);
    {
        std::vector<double> M(3 * (size_t)N + H, 0.0);
        for (uint32_t h = 0; h < H; ++h) M[2 * N + h] = P.HJ0[h];
        for (uint32_t i = 0; i < N; ++i) M[2 * N + H + i] = P.off[i];
        c.M = u.put(M);
    }
    c.HJ0 = u.put(P.HJ0);
    c.HS2 = u.put(P.HS2);
    c.CmByDt = u.put(P.CmByDt);
    c.EmByRm = u.put(P.EmByRm);
    c.injBasal = u.put(P.injBasal);
    c.injVarying = u.zeros<double>(N);
    c.ext = u.zeros<double>(2 * (size_t)N);
    c.prevExt = u.zeros<double>(2 * (size_t)N);
    c.chanPtr = u.put(P.chanPtr);
    c.poolPtr = u.put(P.poolPtr);
    c.extPtr = u.put(P.extPtr);
    c.extList = u.put(P.extList);
    c.fLevelPtr = u.put(P.fLevelPtr);
    c.fRows = u.put(P.fRows);
    c.fOpPtr = u.put(P.fOpPtr);
    c.fOps = reinterpret_cast<const int4*>(u.put(P.fOps));
    c.bLevelPtr = u.put(P.bLevelPtr);
    c.bRows = u.put(P.bRows);
    c.bTermPtr = u.put(P.bTermPtr);
    c.bTerms = reinterpret_cast<const int2*>(u.put(P.bTerms));
    c.fRun = u.put(P.fRun);
    c.fRunRow = u.put(P.fRunRow);
    c.bRun = u.put(P.bRun);
    c.bRunRow = u.put(P.bRunRow);
    c.fWaves = P.fWavePtr.empty() ? 0 : (uint32_t)P.fWavePtr.size() - 1;
    c.fWavePtr = u.put(P.fWavePtr);
    c.fWaveOps = reinterpret_cast<const int4*>(u.put(P.fWaveOps));
    c.Gbar = u.put(P.Gbar);
    c.Ek = u.put(P.Ek);
    c.Xpow = u.put(P.Xpow);
    c.Ypow = u.put(P.Ypow);
    c.Zpow = u.put(P.Zpow);
    c.mod = u.put(P.modulation);
    c.Gk = u.zeros<double>(P.C);
    c.state = u.put(P.state0);
    c.extCa = u.zeros<double>(P.C);
    c.instant = u.put(P.instant);
    c.stateOff = u.put(P.stateOff);
    c.colX = u.put(P.colX);
    c.colY = u.put(P.colY);
    c.colZ = u.put(P.colZ);
    c.zSrc = u.put(P.zSrc);
    {
        std::vector<uint32_t> cc(P.C);
        for (uint32_t ic = 0; ic < N; ++ic)
            for (uint32_t q = P.chanPtr[ic]; q < P.chanPtr[ic + 1]; ++q) cc[q] = ic;
        c.chanCompt = u.put(cc);
    }
    c.c = u.put(P.c0);
    c.CaBasal = u.put(P.CaBasal);
    c.f1 = u.put(P.f1);
    c.f2 = u.put(P.f2);
    c.ceil = u.put(P.ceiling);
    c.floor_ = u.put(P.floor_);
    c.ca = u.zeros<double>(P.P);
    c.iCa = u.zeros<double>(P.P);
    c.feedPtr = u.put(P.feedPtr);
    c.feedChan = u.put(P.feedChan);
    c.vTab = sh ? sh->vTab : u.put(P.vTable.data);
    c.vCol = P.vTable.nCol; c.vMin = P.vTable.min; c.vMax = P.vTable.max; c.vDx = P.vTable.dx;
    c.caTab = sh ? sh->caTab : u.put(P.caTable.data);
    c.caCol = P.caTable.nCol; c.caMin = P.caTable.min; c.caMax = P.caTable.max; c.caDx = P.caTable.dx;
    {
        std::vector<double> AB, geom;
        std::vector<uint64_t> off;
        std::vector<uint32_t> nn;
        for (const Gate2D& g : P.gates2d) {
            if (!sh) {
                off.push_back(AB.size());
                AB.insert(AB.end(), g.AB.begin(), g.AB.end());
            }
            geom.insert(geom.end(), {g.xmin, g.xmax, g.ymin, g.ymax, g.invDx, g.invDy});
            nn.push_back(g.nx);
            nn.push_back(g.ny);
        }
        if (sh) {
            c.g2dAB = sh->g2dBase;
            c.g2dOff = u.put(sh->g2dOff);
        } else {
            c.g2dAB = u.put(AB);
            c.g2dOff = u.put(off);
        }
        c.g2dGeom = u.put(geom);
        c.g2dN = u.put(nn);
    }
    c.c2dCompt = u.put(P.c2dCompt);
    c.c2dGate = u.put(P.c2dGate);
    c.c2dDep0 = u.put(P.c2dDep0);
    c.c2dDep1 = u.put(P.c2dDep1);
    c.c2dConc1 = u.put(P.c2dConc1);
    c.c2dConc2 = u.put(P.c2dConc2);
    c.c2dInstant = u.put(P.c2dInstant);
    c.c2dGbar = u.put(P.c2dGbar);
    c.c2dEk = u.put(P.c2dEk);
    c.c2dXpow = u.put(P.c2dXpow);
    c.c2dMod = u.put(P.c2dMod);
    c.c2dX = u.put(P.c2dX0);
    c.c2dGk = u.zeros<double>(P.K2);
    c.c2dVm = u.zeros<double>(P.K2);
    c.c2dC1 = u.zeros<double>(P.K2);
    c.c2dC2 = u.zeros<double>(P.K2);
    c.synCompt = u.put(P.synCompt);
    c.synEk = u.put(P.synEk);
    c.synMod = u.put(P.synMod);
    c.synX = u.zeros<double>(P.S);
    c.synY = u.zeros<double>(P.S);
    c.synAct = u.zeros<double>(P.S);
    c.synGk = u.zeros<double>(P.S);
    c.synXc1 = u.zeros<double>(P.S);
    c.synXc2 = u.zeros<double>(P.S);
    c.synYc1 = u.zeros<double>(P.S);
    c.synYc2 = u.zeros<double>(P.S);
    c.synNorm = u.zeros<double>(P.S);
    c.evPtr = u.put(P.evPtr);
    c.evCur = u.put(P.evPtr);
    c.evTime = u.put(P.evTime);
    c.evW = u.put(P.evW);
    c.sgCompt = u.put(P.sgCompt);
    c.sgThreshold = u.put(P.sgThreshold);
    c.sgRefract = u.put(P.sgRefract);
    c.sgLast = u.zeros<double>(P.SG);
    c.sgEdge = u.put(P.sgEdge);
    c.sgFired = u.zeros<int32_t>(P.SG);
    c.spikeCap = spikeCap;
    c.spikeGen = u.zeros<uint32_t>(spikeCap);
    c.spikeTime = u.zeros<double>(spikeCap);
    c.stimStep = u.put(P.stimStep);
    c.stimCompt = u.put(P.stimCompt);
    c.stimValue = u.put(P.stimValue);
    c.injPresent = u.put(P.injPresent);
    c.nDif = P.nDif;
    if (P.nDif) {
        c.difKind = u.put(P.difKind);
        c.difPar = u.put(P.difPar);
        c.difOff = u.put(P.difOff);
        c.difDst = u.put(P.difDst);
        c.ikOff = u.put(P.ikOff);
        c.ikDst = u.put(P.ikDst);
        // state; a DifBuffer starts from its activation field
        std::vector<double> st((size_t)kDifState * P.nDif, 0.0);
        for (uint32_t k = 0; k < P.nDif; ++k)
            if (P.difKind[k] == HS_DIF_BUFFER) st[9 * (size_t)P.nDif + k] = P.difPar[(size_t)k * HS_DIF_NPAR + 11];
        c.difState = u.put(st);
    }
    c.nRec = 0;
    c.recStride = 1;
    c.recCap = 0;
    c.recLd = 0;
    c.ctl = u.zeros<DevCtl>(1);
    return u.err;
}

void synConsts(const CellPlan& P, double dt, double* out) {
    for (uint32_t k = 0; k < P.S; ++k)
        synchanConstants(P.synTau1[k], P.synTau2[k], P.synGbar[k], dt, out + 5 * k, out + 5 * k + 1,
                         out + 5 * k + 2, out + 5 * k + 3, out + 5 * k + 4);
}

}  // namespace hsg
