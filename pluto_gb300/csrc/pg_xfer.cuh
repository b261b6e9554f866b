// Host <-> device transfers of one state array with the device reading or
// writing the host array in place: pinned (mapped) host memory through its
// device alias, and pageable memory where the device walks the host's page
// tables (address translation over NVLink-C2C on Grace).  One kernel moves
// the array and applies the layout mapping and, for FP32 device storage, the
// conversion; no device staging copy, no per-array synchronisation.  Other
// host memory takes the copy-engine path of the caller.
#pragma once
#include "pg_internal.h"
#include "pg_dw.cuh"

namespace pg {

// Host extents of one array and the device offset (device index = host index
// + off) for the two layouts of pg_upload / pg_download:
//   PG_LAYOUT_INTERIOR: the interior box; a face array is one longer along
//                       its axis and starts at the face beg-1
//   PG_LAYOUT_PLUTO   : the whole ghosted array; a face array is one longer
//                       along its axis with the -1 layer first, which the
//                       device arrays do not store (skipped)
struct HostBox {
  int hn[3], off[3];
};

inline HostBox host_box(const Geom& g, int fd, int layout) {
  HostBox b;
  for (int ax = 0; ax < 3; ax++) {
    const bool st = ax == fd && ax < g.dims;
    if (layout == PG_LAYOUT_PLUTO) {
      b.hn[ax] = g.nt[ax] + (st ? 1 : 0);
      b.off[ax] = st ? -1 : 0;
    } else {
      b.hn[ax] = g.nx[ax] + (st ? 1 : 0);
      b.off[ax] = g.beg[ax] - (st ? 1 : 0);
    }
  }
  return b;
}

__device__ __forceinline__ void host_to_dev(double v, float* d) { *d = narrow(v); }
__device__ __forceinline__ void host_to_dev(double v, double* d) { *d = v; }
__device__ __forceinline__ double dev_to_host(float v) { return widen(v); }
__device__ __forceinline__ double dev_to_host(double v) { return v; }

template <class D>
__global__ void k_host_xfer(double* host, D* dev, Geom g, HostBox b, int to_dev) {
  const long long n = (long long)b.hn[0] * b.hn[1] * b.hn[2];
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += stride) {
    const int x = (int)(q % b.hn[0]);
    const long long r = q / b.hn[0];
    const int y = (int)(r % b.hn[1]), z = (int)(r / b.hn[1]);
    const int i = x + b.off[0], j = y + b.off[1], k = z + b.off[2];
    if (i < 0 || j < 0 || k < 0) continue;
    const long long c = cidx(g, k, j, i);
    if (to_dev) host_to_dev(host[q], dev + c);
    else host[q] = dev_to_host(dev[c]);
  }
}

// Device-usable address of a host array, or nullptr when the device cannot
// reach it directly (then the caller copies through the copy engines).
inline double* host_alias(const void* h) {
  if (!h) return nullptr;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, h) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (at.type == cudaMemoryTypeHost && at.devicePointer) return (double*)at.devicePointer;
  if (at.type == cudaMemoryTypeUnregistered) {
    int dev = 0, ats = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&ats, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) == cudaSuccess &&
        ats == 1)
      return (double*)h;
    cudaGetLastError();
  }
  return nullptr;
}

template <class D>
inline void launch_host_xfer(cudaStream_t st, double* alias, D* dev, const Geom& g, int fd, int layout,
                             bool to_dev) {
  int dv = 0, nsm = 152;
  if (cudaGetDevice(&dv) == cudaSuccess) cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dv);
  const HostBox b = host_box(g, fd, layout);
  const long long n = (long long)b.hn[0] * b.hn[1] * b.hn[2];
  long long blocks = (n + 255) / 256;
  if (blocks > 8LL * nsm) blocks = 8LL * nsm;
  if (blocks < 1) blocks = 1;
  k_host_xfer<D><<<(unsigned)blocks, 256, 0, st>>>(alias, dev, g, b, to_dev ? 1 : 0);
}

}  // namespace pg
