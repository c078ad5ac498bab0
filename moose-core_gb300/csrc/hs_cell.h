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
cudaError_t layoutCell(const CellPlan& P, Arena& a, DevCell& dc, uint32_t spikeCap,
                       uint32_t recCap, uint32_t nRec, cudaStream_t st,
                       std::vector<void*>* pinnedKeep);

// Host-side reinit of one cell's device state (HSolveActive::reinit plus the
// tick-1/4 objects' reinit); gates are set by the reinit kernel afterwards.
cudaError_t reinitCellState(const CellPlan& P, const DevCell& dc, double clockDt,
                            const std::vector<double>& initVm, const std::vector<double>& injBasal,
                            const std::vector<uint8_t>& injPresent, cudaStream_t st);

cudaError_t launchStepFp64(const DevCell& c, uint32_t nsteps, cudaStream_t st);
cudaError_t launchReinitGatesFp64(const DevCell& c, cudaStream_t st);

}  // namespace hsg
