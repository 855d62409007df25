// pd_noalloc.cu -- pd_count_live_bonds_noalloc: the live-bond count without any device
// allocation.
//
// pd_count_live_bonds allocates a device accumulator with cudaMalloc on every call. Some
// callers cannot do that: a progress monitor that polls a running simulation from a host
// callback or another thread must not allocate, because cudaMalloc synchronises the whole
// device and would stall the step pipeline it is watching; an application that hands all free
// HBM to resident simulations (or that runs under a framework owning the allocator) may have
// no free memory to allocate from. This entry point keeps its scratch in a file-scope
// static __device__ array instead, so it allocates nothing.
//
// Limits and sharing: the scratch holds one partial sum per block of 256 nodes plus the
// total, for at most kNoAllocMaxNodes = 1,048,576 nodes; larger simulations are rejected with
// PD_EINVAL. Every GPU that loads the library holds this 32 KB array until the process exits.
// All calls on a device share the array and it keeps the last call's contents; each call
// overwrites every slot it reads, so nothing needs clearing, but calls whose kernels overlap on
// the GPU (different streams or threads at the same time) race on it.
//
// Set-up: the first call on a device looks up the array's device address with
// cudaGetSymbolAddress while that device is current and remembers it for that device. That
// first call should come before any stream capture. Every call runs on the simulation's own
// device (the device of its stream): when another device is current, the call makes the
// simulation's device current for its duration and restores the caller's device afterwards.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "pd_engine.h"
#include "pd_sim.h"

namespace pdg {
namespace {

constexpr int kNoAllocThreads = 256;
constexpr uint32_t kNoAllocMaxBlocks = 4096;
constexpr uint64_t kNoAllocMaxNodes = (uint64_t)kNoAllocThreads * kNoAllocMaxBlocks;
constexpr int kMaxDevices = 64;

// [0, kNoAllocMaxBlocks): per-block partial counts; [kNoAllocMaxBlocks]: the total
static __device__ __align__(256) unsigned long long g_live_scratch[kNoAllocMaxBlocks + 1];

std::mutex g_setup_mutex;
unsigned long long *g_scratch_addr[kMaxDevices] = {};

// Per-block partial count of live bits of movable particles' rows (written unconditionally).
__global__ void __launch_bounds__(kNoAllocThreads) k_live_partials(DevView v, unsigned long long *part) {
  __shared__ unsigned long long warp_sums[kNoAllocThreads / 32];
  const uint64_t n = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long c = 0;
  if (n < v.N && v.parts[v.pid[n]].movable) {
    const uint32_t lane = (uint32_t)(n & 31);
    const uint64_t mbase = v.slice_ptr[n >> 5] >> 5;
    const int dg = v.deg[n];
    for (int j = 0; j < dg; ++j) c += (v.mask[mbase + j] >> lane) & 1u;
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int w = 0; w < kNoAllocThreads / 32; ++w) t += warp_sums[w];
    part[blockIdx.x] = t;
  }
}

// Sum of the partials in block order into part[kNoAllocMaxBlocks].
__global__ void k_live_total(unsigned long long *part, uint32_t nblocks) {
  __shared__ unsigned long long sums[kNoAllocThreads];
  unsigned long long t = 0;
  for (uint32_t b = threadIdx.x; b < nblocks; b += blockDim.x) t += part[b];
  sums[threadIdx.x] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long tot = 0;
    for (int i = 0; i < kNoAllocThreads; ++i) tot += sums[i];
    part[kNoAllocMaxBlocks] = tot;
  }
}

}  // namespace
}  // namespace pdg

namespace {
int count_on_device(pd_sim *s, cudaStream_t st, int dev, uint64_t N, uint64_t *live);
}

extern "C" int pd_count_live_bonds_noalloc(pd_sim *s, uint64_t *live) {
  using namespace pdg;
  if (!s || !live) return PD_EINVAL;
  const uint64_t N = s->eng.num_nodes();
  if (N > kNoAllocMaxNodes) {
    s->eng.err = "pd_count_live_bonds_noalloc: " + std::to_string(N) + " nodes exceed the static scratch limit of " +
                 std::to_string(kNoAllocMaxNodes) + " nodes";
    return PD_EINVAL;
  }
  if (N == 0) {  // nothing to count (and no zero-block launch)
    *live = 0;
    return PD_OK;
  }
  cudaStream_t st = s->eng.stream();
  int dev = 0, caller_dev = 0;
  cudaError_t e = cudaStreamGetDevice(st, &dev);
  if (e == cudaSuccess) e = cudaGetDevice(&caller_dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    s->eng.err = "pd_count_live_bonds_noalloc: no usable device for the simulation's stream";
    return PD_ECUDA;
  }
  if (caller_dev != dev && cudaSetDevice(dev) != cudaSuccess) {
    s->eng.err = "pd_count_live_bonds_noalloc: cannot make the simulation's device current";
    return PD_ECUDA;
  }
  const int rc = count_on_device(s, st, dev, N, live);
  if (caller_dev != dev) cudaSetDevice(caller_dev);
  return rc;
}

namespace {
// The count itself, with the simulation's device current.
int count_on_device(pd_sim *s, cudaStream_t st, int dev, uint64_t N, uint64_t *live) {
  using namespace pdg;
  cudaError_t e = cudaSuccess;
  unsigned long long *scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
      void *p = nullptr;
      e = cudaGetSymbolAddress(&p, g_live_scratch);
      if (e != cudaSuccess || !p) {
        s->eng.err = std::string("pd_count_live_bonds_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e);
        return PD_ECUDA;
      }
      g_scratch_addr[dev] = static_cast<unsigned long long *>(p);
    }
    scratch = g_scratch_addr[dev];
  }
  const uint32_t nblocks = (uint32_t)((N + kNoAllocThreads - 1) / kNoAllocThreads);
  k_live_partials<<<nblocks, kNoAllocThreads, 0, st>>>(s->eng.current_view(), scratch);
  k_live_total<<<1, kNoAllocThreads, 0, st>>>(scratch, nblocks);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    s->eng.err = std::string("pd_count_live_bonds_noalloc: launch: ") + cudaGetErrorString(e);
    return PD_ECUDA;
  }
  unsigned long long h = 0;
  e = cudaMemcpyAsync(&h, scratch + kNoAllocMaxBlocks, sizeof(h), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    s->eng.err = std::string("pd_count_live_bonds_noalloc: ") + cudaGetErrorString(e);
    return PD_ECUDA;
  }
  *live = h;
  return PD_OK;
}
}  // namespace
