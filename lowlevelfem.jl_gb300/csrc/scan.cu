// Device-wide exclusive prefix sum of int64 counts (pattern offsets, CSC
// column pointers).  Three phases: per-block scan of 2048-element tiles, a
// recursive scan of the tile totals, and a uniform add of the tile offsets.
#include "common.cuh"

namespace {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__global__ void k_scan_tiles(const int64_t *__restrict__ in,
                             int64_t *__restrict__ out, int64_t n,
                             int64_t *__restrict__ tile_totals) {
  __shared__ int64_t warp_sums[SCAN_THREADS / 32];
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
  int64_t v[SCAN_ITEMS];
  int64_t local = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    int64_t idx = base + (int64_t)threadIdx.x * SCAN_ITEMS + k;
    v[k] = idx < n ? in[idx] : 0;
    local += v[k];
  }
  // inclusive warp scan of the per-thread totals
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t incl = local;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    int64_t t = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += t;
  }
  if (lane == 31) warp_sums[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int64_t ws = lane < SCAN_THREADS / 32 ? warp_sums[lane] : 0;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      int64_t t = __shfl_up_sync(0xffffffffu, ws, off);
      if (lane >= off) ws += t;
    }
    if (lane < SCAN_THREADS / 32) warp_sums[lane] = ws;  // inclusive
  }
  __syncthreads();
  int64_t run = incl - local + (warp > 0 ? warp_sums[warp - 1] : 0);
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    int64_t idx = base + (int64_t)threadIdx.x * SCAN_ITEMS + k;
    if (idx < n) out[idx] = run;
    run += v[k];
  }
  if (threadIdx.x == SCAN_THREADS - 1) tile_totals[blockIdx.x] = run;
}

__global__ void k_scan_add(int64_t *__restrict__ out, int64_t n,
                           const int64_t *__restrict__ tile_offsets) {
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
  const int64_t add = tile_offsets[blockIdx.x];
  for (int k = threadIdx.x; k < SCAN_TILE; k += SCAN_THREADS) {
    int64_t idx = base + k;
    if (idx < n) out[idx] += add;
  }
}

cudaError_t scan_rec(llf_ctx *ctx, const int64_t *in, int64_t *out, int64_t n,
                     int64_t *d_total) {
  cudaStream_t s = ctx->stream;
  ctx->allocs += 2;
  int64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (tiles < 1) tiles = 1;
  int64_t *totals = nullptr, *offs = nullptr;
  cudaError_t e = cudaMallocAsync((void **)&totals, sizeof(int64_t) * (tiles + 1), s);
  if (e != cudaSuccess) return e;
  e = cudaMallocAsync((void **)&offs, sizeof(int64_t) * (tiles + 1), s);
  if (e != cudaSuccess) return e;
  k_scan_tiles<<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(in, out, n, totals);
  if (tiles > 1) {
    e = scan_rec(ctx, totals, offs, tiles, d_total);
    if (e != cudaSuccess) return e;
    k_scan_add<<<(unsigned)tiles, SCAN_THREADS, 0, s>>>(out, n, offs);
  } else {
    cudaMemcpyAsync(d_total, totals, sizeof(int64_t), cudaMemcpyDeviceToDevice, s);
  }
  cudaFreeAsync(totals, s);
  cudaFreeAsync(offs, s);
  return cudaGetLastError();
}

}  // namespace

// out[i] = sum_{k<i} in[k]; *d_total (device) receives the sum of all n
// inputs; nothing synchronises.
cudaError_t exclusive_scan_i64_dev(llf_ctx *ctx, const int64_t *in, int64_t *out, int64_t n, int64_t *d_total) {
  cudaError_t e = cudaMemsetAsync(d_total, 0, sizeof(int64_t), ctx->stream);
  if (e != cudaSuccess) return e;
  if (n > 0) return scan_rec(ctx, in, out, n, d_total);
  return cudaGetLastError();
}

// out[i] = sum_{k<i} in[k]; *total_host (if non-null) receives the sum of all
// n inputs (synchronising the stream).  in may equal out.
cudaError_t exclusive_scan_i64(llf_ctx *ctx, const int64_t *in, int64_t *out,
                               int64_t n, int64_t *total_host) {
  int64_t *d_total = nullptr;
  ctx->allocs++;
  cudaError_t e = cudaMallocAsync((void **)&d_total, sizeof(int64_t), ctx->stream);
  if (e != cudaSuccess) return e;
  cudaMemsetAsync(d_total, 0, sizeof(int64_t), ctx->stream);
  if (n > 0) {
    e = scan_rec(ctx, in, out, n, d_total);
    if (e != cudaSuccess) return e;
  }
  if (total_host) {
    e = cudaMemcpyAsync(total_host, d_total, sizeof(int64_t), cudaMemcpyDeviceToHost,
                        ctx->stream);
    if (e != cudaSuccess) return e;
    e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return e;
  }
  cudaFreeAsync(d_total, ctx->stream);
  return cudaGetLastError();
}
