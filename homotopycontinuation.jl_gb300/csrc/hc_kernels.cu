// hc_kernels.cu — the library's instantiations of the path-tracking kernel
// (hc_track_kernel.cuh), the batch kernel over many homotopies, and their host launchers.
#include "hc_track_kernel.cuh"

namespace hcd {

// Batch kernel: shared memory = [Launch of the current unit][tables][warp 0][warp 1]...
// Per unit: thread 0 takes the next unit and writes its Launch, all threads stage the
// instance's tables, warps track the unit's paths, and a barrier closes the unit before the
// tables are overwritten. Paths are numbered within their instance (path_number = k + 1).
template <bool MIXED>
__global__ void __launch_bounds__(HC_MAX_BATCH_WARPS * 32) track_batch_kernel(const __grid_constant__ BatchLaunch bl) {
  extern __shared__ __align__(16) char smem[];
  __shared__ int s_unit;
  __shared__ unsigned s_next;
  Launch* la = (Launch*)smem;
  char* tbase = smem + HC_LAUNCH_SMEM;
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  char* wbase = tbase + bl.tbytes + (size_t)wib * bl.wstride;
  PathTracker<MIXED>* T = (PathTracker<MIXED>*)wbase;  // WarpLayout::state == 0 for every instance
  T->reset_counters();
  unsigned long long npaths_done = 0;
  while (true) {
    __syncthreads();  // the previous unit is closed
    if (threadIdx.x == 0) {
      int u = (int)atomicAdd(bl.base.counter, 1ULL);
      s_unit = u;
      s_next = 0;
      if (u < bl.nunits) {
        const BatchInstance& I = bl.inst[bl.units[u].inst];
        *la = bl.base;
        la->P = I.P;
        la->T = I.T;
        la->L = I.L;
        la->npaths = I.npaths;
        la->starts = bl.base.starts + I.vec_off;
        la->res = bl.base.res + I.path_off;
        la->sol = bl.base.sol + I.vec_off;
        la->val = bl.base.val ? bl.base.val + I.vec_off : nullptr;
        la->last = bl.base.last ? bl.base.last + I.vec_off : nullptr;
      }
    }
    __syncthreads();
    const int u = s_unit;
    if (u >= bl.nunits) break;
    const BatchUnit U = bl.units[u];
    const TableLayout& TL = la->T;
    stage(tbase + TL.vcoef64, la->P.vcoef64, TL.n64);
    if (MIXED) stage(tbase + TL.vcoef32, la->P.vcoef32, TL.n32);
    stage(tbase + TL.vmono, la->P.vmono, TL.nmono);
    stage(tbase + TL.jcode, la->P.jcode, TL.njcode);
    stage(tbase + TL.mdef, la->P.mdef, TL.nmdef);
    __syncthreads();
    T->init(la, wbase, tbase);
    __syncwarp();
    auto take = [&](int64_t& kk) -> bool {  // the next path of the unit
      unsigned k = 0;
      if (lane == 0) k = atomicAdd(&s_next, 1u);
      k = __shfl_sync(FULL, k, 0);
      kk = (int64_t)U.lo + k;
      return kk < U.hi;
    };
    auto cancel_result = [&](int64_t kk) {
      if (lane == 0) {
        hc_path_result R;
        memset(&R, 0, sizeof(R));
        R.path_number = kk + 1;
        R.return_code = la->mode == 1 ? EC_terminated_unknown : TC_terminated_unknown;
        la->res[kk] = R;
      }
    };
    if (!bl.base.lockstep) {
      int64_t kk;
      while (take(kk)) {
        if (T->cancelled()) {
          cancel_result(kk);
          continue;
        }
        T->run(kk);
        ++npaths_done;
      }
    } else {
      // lockstep within the unit (see track_kernel): one step per warp per round, then a barrier
      // of the CTA or of the warps sharing a sub-partition; the unit closes at the barrier above
      bool active = false, done = false;
      int64_t kk = 0;
      while (true) {
        if (!active && !done) {
          if (!take(kk)) {
            done = true;
          } else if (T->cancelled()) {
            cancel_result(kk);
          } else {
            T->begin(kk);
            active = T->tracking();
            if (!active) {
              T->finish(kk);
              ++npaths_done;
            }
          }
        } else if (active && !T->step()) {
          T->finish(kk);
          active = false;
          ++npaths_done;
        }
        if (lockstep_round(bl.base.lockstep, done && !active)) break;
      }
    }
  }
  __syncwarp();
  if (lane == 0 && bl.base.stats) add_stats(bl.base.stats, T, npaths_done);
  if (lane == 0) add_phases(bl.base.phase, T);
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

cudaError_t prepare_batch(int precision, size_t smem, int warps_per_cta, int* blocks_per_sm) {
  cudaError_t e;
  if (precision == HC_PREC_MIXED) {
    e = cudaFuncSetAttribute(track_batch_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, track_batch_kernel<true>, 32 * warps_per_cta,
                                                        smem);
  } else {
    e = cudaFuncSetAttribute(track_batch_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, track_batch_kernel<false>,
                                                        32 * warps_per_cta, smem);
  }
  return e;
}

// launch only (prepare_batch sets the shared-memory attribute first, outside stream capture)
cudaError_t launch_batch(const BatchLaunch& bl, int blocks, int warps_per_cta, size_t smem, cudaStream_t stream) {
  if (bl.base.O.precision == HC_PREC_MIXED)
    track_batch_kernel<true><<<blocks, 32 * warps_per_cta, smem, stream>>>(bl);
  else
    track_batch_kernel<false><<<blocks, 32 * warps_per_cta, smem, stream>>>(bl);
  return cudaGetLastError();
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
