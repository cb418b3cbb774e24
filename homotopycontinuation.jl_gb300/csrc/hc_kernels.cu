// hc_kernels.cu — the persistent path-tracking kernel. Each CTA first stages the per-term
// coefficient tables of the homotopy in shared memory (16-byte vector copies, shared by all
// its warps); then each warp pulls path indices from a device work queue (one atomic per
// path, the GPU counterpart of threaded_solve's atomic counter, src/solve.jl:641-669) and
// tracks the path to completion with a PathTracker that lives in shared memory.
#include "hc_track.cuh"

namespace hcd {

__device__ __forceinline__ void stage(char* dst, const void* src, int bytes) {
  const uint4* s = (const uint4*)src;
  uint4* d = (uint4*)dst;
  for (int i = threadIdx.x; i < bytes / 16; i += blockDim.x) d[i] = __ldg(s + i);
}

template <bool MIXED>
__global__ void __launch_bounds__(256) track_kernel(const __grid_constant__ Launch la) {
  static_assert(sizeof(PathTracker<MIXED>) <= HC_STATE_BYTES, "tracker state exceeds its shared-memory slot");
  extern __shared__ __align__(16) char smem[];
  const TableLayout& TL = la.T;
  stage(smem + TL.vcoef64, la.P.vcoef64, TL.n64);
  if (MIXED) stage(smem + TL.vcoef32, la.P.vcoef32, TL.n32);
  stage(smem + TL.vmono, la.P.vmono, TL.nmono);
  stage(smem + TL.jcode, la.P.jcode, TL.njcode);
  stage(smem + TL.mdef, la.P.mdef, TL.nmdef);
  __syncthreads();
  const int wib = threadIdx.x >> 5;
  char* wbase = smem + TL.bytes + (size_t)wib * la.L.bytes;
  PathTracker<MIXED>* T = (PathTracker<MIXED>*)(wbase + la.L.state);
  T->init(&la, wbase, smem);
  __syncwarp();
  const int lane = threadIdx.x & 31;
  unsigned long long npaths_done = 0;
  while (true) {
    unsigned long long k = 0;
    if (lane == 0) k = atomicAdd(la.counter, 1ULL);
    k = __shfl_sync(FULL, k, 0);
    if (k >= (unsigned long long)la.npaths) break;
    if (T->cancelled()) {
      if (lane == 0) {
        hc_path_result R;
        memset(&R, 0, sizeof(R));
        R.path_number = k + 1;
        R.return_code = la.mode == 1 ? EC_terminated_unknown : TC_terminated_unknown;
        la.res[k] = R;
      }
      continue;
    }
    T->run((int64_t)k);
    ++npaths_done;
  }
  __syncwarp();
  if (lane == 0 && la.stats) {
    atomicAdd(la.stats + 0, npaths_done);
    atomicAdd(la.stats + 1, T->c_evalj);
    atomicAdd(la.stats + 2, T->c_eval);
    atomicAdd(la.stats + 3, T->c_evaldd);
    atomicAdd(la.stats + 4, T->c_taylor);
    atomicAdd(la.stats + 5, T->c_lu);
    atomicAdd(la.stats + 6, T->c_solve);
    atomicAdd(la.stats + 7, T->c_taylor64);
    atomicAdd(la.stats + 8, T->c_switch64);
  }
}

// host-callable launchers
template <bool MIXED>
static cudaError_t launch_t(const Launch& la, int blocks, int warps_per_cta, size_t smem, cudaStream_t stream) {
  cudaError_t e = cudaFuncSetAttribute(track_kernel<MIXED>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  track_kernel<MIXED><<<blocks, 32 * warps_per_cta, smem, stream>>>(la);
  return cudaGetLastError();
}

cudaError_t launch_track(const Launch& la, int blocks, int warps_per_cta, cudaStream_t stream) {
  size_t smem = (size_t)la.T.bytes + (size_t)warps_per_cta * la.L.bytes;
  if (la.O.precision == HC_PREC_MIXED) return launch_t<true>(la, blocks, warps_per_cta, smem, stream);
  return launch_t<false>(la, blocks, warps_per_cta, smem, stream);
}

cudaError_t occupancy(int precision, int warps_per_cta, size_t smem, int* blocks_per_sm) {
  if (precision == HC_PREC_MIXED) {
    cudaFuncSetAttribute(track_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, track_kernel<true>, 32 * warps_per_cta, smem);
  }
  cudaFuncSetAttribute(track_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, track_kernel<false>, 32 * warps_per_cta, smem);
}

}  // namespace hcd
