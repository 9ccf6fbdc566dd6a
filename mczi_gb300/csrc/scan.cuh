// scan.cuh -- reduce-then-scan over an array of small structs with a
// user-supplied associative combine (used for per-tile summaries, where the
// arrays hold a few thousand to a few million entries).
//
//   Op must provide:  static __device__ T identity();
//                     static __device__ T combine(const T& a, const T& b);  // a before b
//
// exclusive_scan(in, out, n, stream, tmp) writes out[i] = in[0] (+) ... (+) in[i-1]
// and out[n] = total.  tmp must hold ceil(n / SCAN_CHUNK) + 1 elements of T.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace mczi {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_PER_THREAD = 8;
constexpr int SCAN_CHUNK = SCAN_THREADS * SCAN_PER_THREAD;

// shuffle of a small trivially-copyable struct, 32 bits at a time
template <class T>
__device__ __forceinline__ T shfl_up_T(const T& v, int d) {
  static_assert(sizeof(T) % 4 == 0, "scan element must be a multiple of 4 bytes");
  T r;
  const uint32_t* src = reinterpret_cast<const uint32_t*>(&v);
  uint32_t* dst = reinterpret_cast<uint32_t*>(&r);
#pragma unroll
  for (int i = 0; i < (int)(sizeof(T) / 4); i++) dst[i] = __shfl_up_sync(0xffffffffu, src[i], d);
  return r;
}

// Exclusive block scan of one value per thread (warp shuffles, then the warp
// totals) over a block of NT threads; returns this thread's exclusive prefix
// and writes the block total to *total (all threads).  sh needs NT / 32 + 1
// entries.
template <class T, class Op, int NT = SCAN_THREADS>
__device__ T block_exclusive_scan(T v, T* total, T* sh) {
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  constexpr int NW = NT / 32;
  T incl = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const T o = shfl_up_T(incl, d);
    if (lane >= d) incl = Op::combine(o, incl);
  }
  if (lane == 31) sh[wid] = incl;
  __syncthreads();
  if (t == 0) {
    T run = Op::identity();
    for (int w = 0; w < NW; w++) {
      const T x = sh[w];
      sh[w] = run;
      run = Op::combine(run, x);
    }
    sh[NW] = run;
  }
  __syncthreads();
  T excl = shfl_up_T(incl, 1);
  if (lane == 0) excl = Op::identity();
  excl = Op::combine(sh[wid], excl);
  *total = sh[NW];
  __syncthreads();
  return excl;
}

template <class T, class Op>
__global__ void __launch_bounds__(SCAN_THREADS) scan_reduce_kernel(const T* __restrict__ in, uint64_t n,
                                                                    T* __restrict__ block_tot) {
  __shared__ T sh[SCAN_THREADS + 1];
  const uint64_t base = (uint64_t)blockIdx.x * SCAN_CHUNK + (uint64_t)threadIdx.x * SCAN_PER_THREAD;
  T acc = Op::identity();
#pragma unroll
  for (int i = 0; i < SCAN_PER_THREAD; i++) {
    uint64_t j = base + i;
    if (j < n) acc = Op::combine(acc, in[j]);
  }
  T tot;
  block_exclusive_scan<T, Op>(acc, &tot, sh);
  if (threadIdx.x == 0) block_tot[blockIdx.x] = tot;
}

// single block: exclusive scan of nb block totals in place; writes grand total to tot[nb]
template <class T, class Op>
__global__ void __launch_bounds__(SCAN_THREADS) scan_top_kernel(T* __restrict__ tot, uint64_t nb) {
  __shared__ T sh[SCAN_THREADS + 1];
  const uint64_t per = (nb + SCAN_THREADS - 1) / SCAN_THREADS;
  const uint64_t lo = per * threadIdx.x;
  const uint64_t hi = lo + per < nb ? lo + per : nb;
  T acc = Op::identity();
  for (uint64_t j = lo; j < hi; j++) acc = Op::combine(acc, tot[j]);
  T total;
  T run = block_exclusive_scan<T, Op>(acc, &total, sh);
  for (uint64_t j = lo; j < hi; j++) {
    T v = tot[j];
    tot[j] = run;
    run = Op::combine(run, v);
  }
  if (threadIdx.x == 0) tot[nb] = total;
}

template <class T, class Op>
__global__ void __launch_bounds__(SCAN_THREADS) scan_apply_kernel(const T* __restrict__ in, uint64_t n,
                                                                   const T* __restrict__ block_pre,
                                                                   T* __restrict__ out) {
  __shared__ T sh[SCAN_THREADS + 1];
  const uint64_t base = (uint64_t)blockIdx.x * SCAN_CHUNK + (uint64_t)threadIdx.x * SCAN_PER_THREAD;
  T vals[SCAN_PER_THREAD];
  T acc = Op::identity();
#pragma unroll
  for (int i = 0; i < SCAN_PER_THREAD; i++) {
    uint64_t j = base + i;
    vals[i] = (j < n) ? in[j] : Op::identity();
    acc = Op::combine(acc, vals[i]);
  }
  T tot;
  T run = Op::combine(block_pre[blockIdx.x], block_exclusive_scan<T, Op>(acc, &tot, sh));
#pragma unroll
  for (int i = 0; i < SCAN_PER_THREAD; i++) {
    uint64_t j = base + i;
    if (j < n) out[j] = run;
    run = Op::combine(run, vals[i]);
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n] = block_pre[gridDim.x];
}

// Host launcher.  `out` holds n + 1 entries; `tmp` ceil(n/SCAN_CHUNK) + 1.
template <class T, class Op>
void exclusive_scan(const T* in, T* out, uint64_t n, T* tmp, cudaStream_t s) {
  if (n == 0) return;
  const uint64_t nb = (n + SCAN_CHUNK - 1) / SCAN_CHUNK;
  scan_reduce_kernel<T, Op><<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, n, tmp);
  scan_top_kernel<T, Op><<<1, SCAN_THREADS, 0, s>>>(tmp, nb);
  scan_apply_kernel<T, Op><<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, n, tmp, out);
}

}  // namespace mczi
