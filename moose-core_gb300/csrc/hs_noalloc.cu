// hs_noalloc.cu -- inject writes without any memory allocation.
//
// hs_batch_set_inject_at (hs_batch_api.cpp) sets the inject of arbitrary
// (cell, compartment) pairs of a batch between process() calls.  The regular
// path registers the targets first (hs_batch_inject_targets), which allocates
// device scratch for their addresses with cudaMalloc and frees the previous
// one with cudaFree.  Some callers cannot allocate there: a serving loop or
// any driver that keeps other batches running on the same GPU (cudaFree
// waits for the whole device, so every running batch would stall behind it),
// and callers that run with a fixed memory budget.  This file gives them a
// path that uses only fixed storage:
//   * a file-scope host staging array and a file-scope device scratch array
//     (static __device__, 256-byte aligned), both of kInjectWriteMax entries
//     (24 bytes each: 768 KiB apiece);
//   * the device address of the scratch is taken once per device, with that
//     device current, by cudaGetSymbolAddress on the first call that uses the
//     device; that first call should therefore come before any stream
//     capture is begun on the device;
//     the address is kept for the life of the library, so the device's
//     primary context must not be reset (cudaDeviceReset) in between;
//   * nothing in the scratch has to start at zero: a call writes the n
//     entries it uses before its kernel reads them;
//   * the n writes of one call are applied by n independent threads, so a
//     (cell, compartment) pair named twice in one call ends with one of its
//     two values, which one is not defined.
// The storage is shared by every batch of the process: calls are serialised
// by a lock and each returns only after its kernel has finished reading the
// scratch, so calls that overlap in time (from several host threads) wait
// for each other; without that lock they would race on the same storage.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "hs_noalloc.h"

namespace hsg {

static __device__ __align__(256) InjectWrite g_injectScratch[kInjectWriteMax];

namespace {

constexpr int kMaxDevices = 64;

InjectWrite g_injectStaging[kInjectWriteMax];
InjectWrite* g_scratchAddr[kMaxDevices];
std::mutex g_injectLock;

__global__ void hsScatterInjectStatic(const InjectWrite* __restrict__ w, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const InjectWrite x = w[i];
    *x.addr = x.value;
    if (x.flag) *x.flag = 1;
}

}  // namespace

std::mutex& injectStaticLock() { return g_injectLock; }

InjectWrite* injectStaging() { return g_injectStaging; }

// Copies staging entries [0, n) into the device scratch of `device` and
// scatters them on `st`; returns after the kernel has finished.  The caller
// holds injectStaticLock() and has made `device` current.
cudaError_t scatterInjectStatic(int device, uint32_t n, cudaStream_t st) {
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    if (n == 0) return cudaSuccess;
    if (n > kInjectWriteMax) return cudaErrorInvalidValue;
    if (!g_scratchAddr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_injectScratch);
        if (e != cudaSuccess) return e;
        g_scratchAddr[device] = static_cast<InjectWrite*>(p);
    }
    InjectWrite* d = g_scratchAddr[device];
    cudaError_t e = cudaMemcpyAsync(d, g_injectStaging, (size_t)n * sizeof(InjectWrite), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    hsScatterInjectStatic<<<(n + 255) / 256, 256, 0, st>>>(d, n);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(st);
}

}  // namespace hsg
