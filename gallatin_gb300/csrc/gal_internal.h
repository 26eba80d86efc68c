// gal_internal.h — functions shared between the library's translation units,
// not part of the C ABI (hidden from the shared library's exported symbols).
#pragma once

#include <cuda_runtime.h>

#include "../../include/gallatin_gb300.h"
#include "../../include/gallatin_gb300/gal_device.cuh"

#define GAL_INTERNAL __attribute__((visibility("hidden")))

// device the handle's allocator lives on
GAL_INTERNAL int gal_internal_device(const gal_handle *h);
// host copy of the device-resident state (array addresses, geometry)
GAL_INTERNAL const gal::state *gal_internal_host_state(const gal_handle *h);

// Makes `device` current for the lifetime of the guard when it is not the
// current one already, and restores the caller's device afterwards.
struct gal_device_guard {
  int prev = -1;
  cudaError_t err = cudaSuccess;
  explicit gal_device_guard(int device) {
    int cur = 0;
    err = cudaGetDevice(&cur);
    if (err == cudaSuccess && cur != device) {
      err = cudaSetDevice(device);
      if (err == cudaSuccess) prev = cur;
    }
  }
  ~gal_device_guard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

// Set-up of the allocation-free export on `device` (gal_noalloc.cu): resolves
// the device address of its fixed staging array (which loads the module that
// holds the array, so the array is placed on the device now) and creates the
// export's own stream.  Called by gal_create with the handle's device
// current; returns GAL_OK or GAL_ERR_CUDA.
GAL_INTERNAL int gal_noalloc_setup(int device);
