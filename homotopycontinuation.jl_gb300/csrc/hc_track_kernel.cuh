// hc_track_kernel.cuh — the persistent path-tracking kernel, shared by the library's own
// translation unit (hc_kernels.cu) and the per-system kernels compiled at run time by NVRTC
// (hc_slp.cu). Each CTA first stages the per-term coefficient tables of the homotopy in
// shared memory (16-byte vector copies, shared by all its warps); then each warp pulls path
// indices from a device work queue (one atomic per path, the GPU counterpart of
// threaded_solve's atomic counter, src/solve.jl:641-669) and tracks the path to completion
// with a PathTracker that lives in shared memory.
#pragma once
#include "hc_track.cuh"

namespace hcd {

__device__ __forceinline__ void stage(char* dst, const void* src, int bytes) {
  const uint4* s = (const uint4*)src;
  uint4* d = (uint4*)dst;
  for (int i = threadIdx.x; i < bytes / 16; i += blockDim.x) d[i] = __ldg(s + i);
}

// End of a lockstep round (hc_options::lockstep): mode 1 waits for the whole CTA; mode 2 for the
// warps that share this warp's SM sub-partition (warps w, w + 4, ...: named barrier 1 + w % 4);
// mode 3 for the warps of sub-partitions {0, 1} or {2, 3} (named barrier 5 or 6). Named barriers
// count 32 threads per member warp. Every participating warp calls it once per round; returns
// true when `done` holds in all of them, so they also leave the loop together.
__device__ __forceinline__ bool lockstep_round(int mode, bool done) {
  if (mode != 2 && mode != 3) return __syncthreads_and(done) != 0;
  const int wib = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int id, members;
  if (mode == 2) {
    const int sub = wib & 3;
    id = 1 + sub;
    members = (nw - sub + 3) >> 2;
  } else {
    const int grp = (wib & 3) >> 1, rem = nw & 3;
    id = 5 + grp;
    members = 2 * (nw >> 2) + (grp == 0 ? (rem < 2 ? rem : 2) : (rem > 2 ? rem - 2 : 0));
  }
  int all;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.s32 p, %1, 0;\n bar.red.and.pred q, %2, %3, p;\n selp.s32 %0, 1, 0, q;\n}"
      : "=r"(all)
      : "r"(done ? 1 : 0), "r"(id), "r"(32 * members)
      : "memory");
  return all != 0;
}

template <bool MIXED>
__device__ __forceinline__ void add_stats(unsigned long long* st, const PathTracker<MIXED>* T,
                                          unsigned long long npaths_done) {
  atomicAdd(st + 0, npaths_done);
  atomicAdd(st + 1, T->c_evalj);
  atomicAdd(st + 2, T->c_eval);
  atomicAdd(st + 3, T->c_evaldd);
  atomicAdd(st + 4, T->c_taylor);
  atomicAdd(st + 5, T->c_lu);
  atomicAdd(st + 6, T->c_solve);
  atomicAdd(st + 7, T->c_taylor64);
  atomicAdd(st + 8, T->c_switch64);
  atomicAdd(st + 9, T->c_learned);
  atomicAdd(st + 10, T->c_learned_rej);
}
template <bool MIXED>
__device__ __forceinline__ void add_phases(unsigned long long* ph, const PathTracker<MIXED>* T) {
#ifdef HC_PHASE_CLOCKS
  if (ph)
    for (int k = 0; k < HC_NPHASE; ++k) atomicAdd(ph + k, T->ph[k]);
#endif
}

template <bool MIXED>
__global__ void __launch_bounds__(HC_MAX_WARPS * 32) track_kernel(const __grid_constant__ Launch la) {
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
  T->reset_counters();
  __syncwarp();
  const int lane = threadIdx.x & 31;
  unsigned long long npaths_done = 0;
  auto take = [&](int64_t& kk) -> bool {  // the next path of the queue; false when it is empty
    unsigned long long k = 0;
    if (lane == 0) k = atomicAdd(la.counter, 1ULL);
    k = __shfl_sync(FULL, k, 0);
    if (k >= (unsigned long long)la.npaths) return false;
    kk = la.path_list ? la.path_list[k] : (int64_t)k;
    return true;
  };
  auto cancel_result = [&](int64_t kk) {
    if (lane == 0) {
      hc_path_result R;
      memset(&R, 0, sizeof(R));
      R.path_number = kk + 1;
      R.return_code = la.mode == 1 ? EC_terminated_unknown : TC_terminated_unknown;
      la.res[kk] = R;
    }
  };
  if (!la.lockstep) {
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
    // lockstep: per round, each warp with a path takes one step of it (a warp without one first
    // takes the next path of the queue and begins it); then the CTA waits for all its warps.
    // Every warp reaches the barrier once per round and all leave together.
    bool active = false, done = false;
    int64_t kk = 0;
#ifdef HC_PHASE_CLOCKS
    const long long t_run = clock64();
#endif
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
#ifdef HC_PHASE_CLOCKS
      const long long t_wait = clock64();
      const bool all_done = lockstep_round(la.lockstep, done && !active);
      if (lane == 0) T->ph[PH_WAIT] += (unsigned long long)(clock64() - t_wait);
      if (all_done) break;
#else
      if (lockstep_round(la.lockstep, done && !active)) break;
#endif
    }
#ifdef HC_PHASE_CLOCKS
    if (lane == 0) T->ph[PH_RUN] += (unsigned long long)(clock64() - t_run);
#endif
  }
  __syncwarp();
  if (lane == 0 && la.stats) add_stats(la.stats, T, npaths_done);
  if (lane == 0) add_phases(la.phase, T);
}

}  // namespace hcd
