// Per-device launch helpers shared by the kernel translation units (sm_103a).
//
// Kernel attributes (dynamic shared memory, carveout) and occupancy are set or queried
// only when a launch asks for more shared memory than before, so that launches enqueued
// during CUDA-graph capture issue no attribute calls (the first, eager launch of each
// kernel instantiation on each device does).  The caches hold kMaxDevices devices; a
// launch on a device with a larger index is refused with LRES_EINVAL.
#pragma once
#include "common.cuh"
#include "../../include/lres_gb300.h"

namespace lres {

constexpr int kMaxDevices = 64;

// Index of the current device, or -1 (error message set) when it is beyond the caches.
static inline int device_slot() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        lres_set_error("device index %d outside the supported range 0..%d", dev, kMaxDevices - 1);
        return -1;
    }
    return dev;
}

template <auto Kern>
static int prepare_kernel(int threads, size_t smem, int* per_sm) {
    static size_t set_smem[kMaxDevices] = {};     // one cache per kernel instantiation and device
    static int cached_per_sm[kMaxDevices] = {};
    static bool done[kMaxDevices] = {};
    const int dev = device_slot();
    if (dev < 0) return LRES_EINVAL;
    if (!done[dev] || smem > set_smem[dev]) {
        LRES_CUDA_TRY(cudaFuncSetAttribute(Kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        // prefer the largest shared-memory carveout, so that the occupancy below is the maximum
        LRES_CUDA_TRY(cudaFuncSetAttribute(Kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                           (int)cudaSharedmemCarveoutMaxShared));
        LRES_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&cached_per_sm[dev], Kern, threads, smem));
        set_smem[dev] = smem;
        done[dev] = true;
    }
    *per_sm = cached_per_sm[dev];
    return LRES_OK;
}

// Multiprocessors of the current device (0 when the device is beyond the caches).
static inline int device_sms() {
    static int nsm[kMaxDevices] = {};
    const int dev = device_slot();
    if (dev < 0) return 0;
    if (!nsm[dev]) cudaDeviceGetAttribute(&nsm[dev], cudaDevAttrMultiProcessorCount, dev);
    return nsm[dev];
}

}  // namespace lres
