// hs_cell.h -- upload of a CellPlan into device memory (one arena per
// solver) and the host mirror used by field access.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "hs_device.cuh"
#include "hs_plan.h"

namespace hsg {

// A bump allocator over one device allocation.
struct Arena {
    char* base = nullptr;
    size_t size = 0, used = 0;
    template <class T>
    T* take(size_t n) {
        size_t off = (used + 255) & ~size_t(255);
        used = off + n * sizeof(T);
        return base ? reinterpret_cast<T*>(base + off) : nullptr;
    }
};

// Lays out (dry run with base == nullptr to size the arena) and uploads one
// cell; fills `dc`.  Static arrays are copied with cudaMemcpyAsync on `st`.
// A batch passes `shared`: device arrays it owns (initVm and SynChan
// constants of all cells contiguous, for one-copy reinit) and rate tables
// shared by the cells that have identical ones.
struct CellShared {
    double* initVm = nullptr;
    double* synConst = nullptr;
    const double* vTab = nullptr;
    const double* caTab = nullptr;
    const double* g2dBase = nullptr;
    std::vector<uint64_t> g2dOff;    // per gate2d of the cell, offset from g2dBase
};
cudaError_t layoutCell(const CellPlan& P, Arena& a, DevCell& dc, uint32_t spikeCap,
                       cudaStream_t st, const CellShared* shared = nullptr);

// SynChan reinit constants of one cell at the clock dt, 5 per SynChan
// (xc1, xc2, yc1, yc2, norm), computed with the host libm as the reference does.
void synConsts(const CellPlan& P, double dt, double* out);

cudaError_t launchStepFp64(const DevCell& c, uint32_t nsteps, cudaStream_t st);
cudaError_t launchStepFp64Cluster(const DevCell& c, uint32_t ctas, uint32_t nsteps, cudaStream_t st);
cudaError_t launchGroupStepFp64(const DevCell* cells, uint32_t n, uint32_t ctas, uint32_t nsteps,
                                cudaStream_t st);
// The queued field writes of a drop-in solver, one thread each (distinct
// addresses).
cudaError_t launchScatterFields(const FieldWrite* w, uint32_t n, cudaStream_t st);
// HSolveActive::reinit + tick-1/4 object reinit of `nCells` cells, on device.
cudaError_t launchReinitFp64(const DevCell* cells, uint32_t nCells, cudaStream_t st);
// Spike read-back of a batch: per-cell counts (FP64 batch), then the stored
// spikes of every cell gathered at off[c] .. off[c+1] (FP64: from `cells`;
// mixed: `cells` null, from the [cell][cap] arrays srcGen/srcTime).
// out[k] = *src[k] for a gather list of n device addresses (doubles, or
// floats when f32); NaN where src[k] is null.
cudaError_t launchGatherValues(const void* const* src, uint32_t f32, uint64_t n, double* out, cudaStream_t st);
cudaError_t launchSpikeCountsFp64(const DevCell* cells, uint32_t nCells, uint32_t* counts, cudaStream_t st);
cudaError_t launchGatherSpikes(const DevCell* cells, const uint32_t* srcGen, const float* srcTime, uint32_t cap,
                               uint32_t nCells, const uint32_t* off, uint32_t* gen, double* time,
                               cudaStream_t st);
cudaError_t launchBatchStepFp64(const DevCell* cells, const uint32_t* warpCellPtr,
                                const uint32_t* warpCells, uint32_t nWarps, const uint32_t* ctaCellPtr,
                                const uint32_t* ctaCells, uint32_t nsteps, uint32_t threadsPerCta,
                                cudaStream_t st);
// CTAs of the FP64 batch kernel that fit on one SM at once (0 if unknown).
int fp64BatchCtasPerSm(uint32_t threadsPerCta);

}  // namespace hsg
