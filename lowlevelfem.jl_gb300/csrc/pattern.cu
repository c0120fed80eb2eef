// Connectivity conversion, node->element adjacency and the structural CSC
// pattern (build_csc_pattern, src/multifield.jl:2083-2250).
//
// Pattern construction, GB300 form:
//   1. node->element lists: one atomic count per (element, node) slot, a
//      device scan, an atomic fill, then a per-node insertion sort by element
//      index so every list is in element order (the order the gather kernel
//      relies on for its deterministic per-entry sums);
//   2. node adjacency: one warp per node gathers the node tags of all its
//      elements into a shared-memory buffer, bitonic-sorts it and keeps the
//      unique tags (count pass, scan, fill pass);
//   3. DoF-level column pointers follow in closed form from the node-level
//      pattern: colptr[p*B+j] = p^2*nptr[B] + j*p*deg(B).
// The DoF-level row indices are never materialised: every consumer derives
// them from the node-level rows (row = p*A + i).
#include "common.cuh"

namespace {

__global__ void k_conn_convert(const int64_t *__restrict__ in,
                               int32_t *__restrict__ out, int64_t count,
                               int64_t non, unsigned *status) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (; i < count; i += stride) {
    int64_t t = in[i];
    if (t < 1 || t > non) {
      atomicOr(status, ST_BAD_NODE);
      out[i] = 0;
    } else {
      out[i] = (int32_t)(t - 1);
    }
  }
}

__global__ void k_check_finite(const double *__restrict__ a, int64_t n,
                               unsigned *status) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  bool bad = false;
  for (; i < n; i += stride) bad |= !isfinite(a[i]);
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(status, ST_NONFINITE);
}

__global__ void k_n2e_count(const int32_t *__restrict__ conn,
                            const int32_t *__restrict__ emat, int64_t nel,
                            int npe, int64_t *__restrict__ cnt) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (; i < nel * npe; i += stride) {
    int64_t e = i / npe;
    if (emat && emat[e] < 0) continue;
    atomicAdd((unsigned long long *)&cnt[conn[i]], 1ull);
  }
}

__global__ void k_n2e_fill(const int32_t *__restrict__ conn,
                           const int32_t *__restrict__ emat, int64_t nel,
                           int npe, const int64_t *__restrict__ ptr,
                           int64_t *__restrict__ cursor, int2 *__restrict__ n2e) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (; i < nel * npe; i += stride) {
    int64_t e = i / npe;
    if (emat && emat[e] < 0) continue;
    int node = conn[i];
    unsigned long long slot = atomicAdd((unsigned long long *)&cursor[node], 1ull);
    n2e[ptr[node] + (int64_t)slot] = make_int2((int)e, (int)(i - e * npe));
  }
}

// Sort every node's element list by element index (insertion sort: lists
// are short — at most a few dozen elements share a node).
__global__ void k_n2e_sort(const int64_t *__restrict__ ptr, int2 *__restrict__ n2e,
                           int64_t non, int *max_len) {
  int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int local_max = 0;
  for (; v < non; v += stride) {
    int64_t s = ptr[v], e = ptr[v + 1];
    for (int64_t a = s + 1; a < e; ++a) {
      int2 key = n2e[a];
      int64_t b = a - 1;
      while (b >= s && n2e[b].x > key.x) {
        n2e[b + 1] = n2e[b];
        --b;
      }
      n2e[b + 1] = key;
    }
    local_max = max(local_max, (int)(e - s));
  }
  atomicMax(max_len, local_max);
}

// One warp per node: collect the node tags of all elements around node B in
// shared memory (cap entries per warp, padded to a power of two), sort,
// count or write the unique tags.
template <bool FILL>
__global__ void k_node_adjacency(const int32_t *__restrict__ conn, int npe,
                                 const int64_t *__restrict__ n2e_ptr,
                                 const int2 *__restrict__ n2e, int64_t non,
                                 int cap, int64_t *__restrict__ deg_or_ptr,
                                 int32_t *__restrict__ nadj,
                                 int32_t *__restrict__ diagpos,
                                 unsigned *status) {
  extern __shared__ int32_t sbuf[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int warps_per_block = blockDim.x >> 5;
  int32_t *buf = sbuf + (size_t)wib * cap;
  int64_t gw = (int64_t)blockIdx.x * warps_per_block + wib;
  int64_t nw = (int64_t)gridDim.x * warps_per_block;
  for (int64_t B = gw; B < non; B += nw) {
    int64_t s = n2e_ptr[B], e = n2e_ptr[B + 1];
    int64_t m = (e - s) * npe;
    if (m > cap) {
      if (lane == 0) atomicOr(status, ST_CAPACITY);
      continue;
    }
    int P = 1;
    while (P < m) P <<= 1;
    for (int t = lane; t < P; t += 32) {
      int32_t val = INT32_MAX;
      if (t < m) {
        int64_t k = s + t / npe;
        int a = t % npe;
        val = conn[(int64_t)n2e[k].x * npe + a];
      }
      buf[t] = val;
    }
    __syncwarp();
    // bitonic sort of buf[0..P)
    for (int k = 2; k <= P; k <<= 1) {
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int t = lane; t < P; t += 32) {
          int partner = t ^ j;
          if (partner > t) {
            int32_t x = buf[t], y = buf[partner];
            bool up = ((t & k) == 0);
            if ((x > y) == up) {
              buf[t] = y;
              buf[partner] = x;
            }
          }
        }
        __syncwarp();
      }
    }
    // unique
    int64_t base = FILL ? deg_or_ptr[B] : 0;
    int count = 0;
    for (int t0 = 0; t0 < m; t0 += 32) {
      int t = t0 + lane;
      bool keep = false;
      int32_t val = 0;
      if (t < m) {
        val = buf[t];
        keep = (t == 0) || (buf[t - 1] != val);
      }
      unsigned bal = __ballot_sync(0xffffffffu, keep);
      if (FILL && keep) {
        int off = count + __popc(bal & ((1u << lane) - 1u));
        nadj[base + off] = val;
        if (val == (int32_t)B) diagpos[B] = off;
      }
      count += __popc(bal);
    }
    if (!FILL && lane == 0) deg_or_ptr[B] = count;
    __syncwarp();
  }
}

__global__ void k_max_deg(const int64_t *__restrict__ deg, int64_t non, int *out) {
  int m = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < non;
       i += (int64_t)gridDim.x * blockDim.x)
    m = max(m, (int)deg[i]);
  atomicMax(out, m);
}

__global__ void k_dof_colptr(const int64_t *__restrict__ nptr, int64_t non,
                             int p, int64_t *__restrict__ colptr) {
  int64_t B = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (; B < non; B += stride) {
    int64_t deg = nptr[B + 1] - nptr[B];
    for (int j = 0; j < p; ++j)
      colptr[B * p + j] = (int64_t)p * p * nptr[B] + (int64_t)j * p * deg;
    if (B == non - 1) colptr[non * p] = (int64_t)p * p * nptr[non];
  }
}

inline unsigned grid_for(int64_t n, int threads, int sms) {
  int64_t b = (n + threads - 1) / threads;
  int64_t cap = (int64_t)sms * 32;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (unsigned)b;
}

}  // namespace

int mesh_convert_conn(llf_ctx *ctx, llf_mesh *mesh, const int64_t *d_conn64) {
  int64_t count = mesh->nel * mesh->npe;
  k_conn_convert<<<grid_for(count, 256, ctx->num_sms), 256, 0, ctx->stream>>>(
      d_conn64, mesh->d_conn, count, mesh->non, ctx->d_status);
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  return LLF_OK;
}

// 1-based tags -> 0-based node indices into out, flagging entries that
// differ from cur.
__global__ void k_conn_update(const int64_t *__restrict__ in, const int32_t *__restrict__ cur,
                              int32_t *__restrict__ out, int64_t count, int64_t non, int *differs,
                              unsigned *status) {
  int d = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = in[i];
    int32_t v = 0;
    if (t < 1 || t > non) atomicOr(status, ST_BAD_NODE);
    else v = (int32_t)(t - 1);
    out[i] = v;
    d |= (v != cur[i]);
  }
  if (__syncthreads_or(d) && threadIdx.x == 0) atomicOr(differs, 1);
}

int mesh_update_conn(llf_ctx *ctx, llf_mesh *mesh, const int64_t *d_conn64, bool *changed) {
  const int64_t count = mesh->nel * mesh->npe;
  int32_t *fresh = nullptr;
  int *d_diff = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &fresh, count));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &d_diff, 1));
  LLF_CUDA_TRY(ctx, cudaMemsetAsync(d_diff, 0, sizeof(int), ctx->stream));
  k_conn_update<<<grid_for(count, 256, ctx->num_sms), 256, 0, ctx->stream>>>(
      d_conn64, mesh->d_conn, fresh, count, mesh->non, d_diff, ctx->d_status);
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  int h = 0;
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(&h, d_diff, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  LLF_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  dfree(ctx, d_diff);
  *changed = h != 0;
  if (*changed) {
    dfree(ctx, mesh->d_conn);
    mesh->d_conn = fresh;
  } else {
    dfree(ctx, fresh);
  }
  return LLF_OK;
}

int check_finite(llf_ctx *ctx, const double *d, int64_t n) {
  if (n <= 0) return LLF_OK;
  k_check_finite<<<grid_for(n, 256, ctx->num_sms), 256, 0, ctx->stream>>>(d, n, ctx->d_status);
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  return LLF_OK;
}

int build_n2e(llf_ctx *ctx, const int32_t *conn, const int32_t *emat, int64_t nel, int npe,
              int64_t non, int64_t **ptr_out, int2 **list_out, int *max_len) {
  cudaStream_t s = ctx->stream;
  int64_t *cnt = nullptr, *ptr = nullptr;
  int2 *list = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &cnt, non + 1));
  LLF_CUDA_TRY(ctx, cudaMemsetAsync(cnt, 0, sizeof(int64_t) * (non + 1), s));
  unsigned g = grid_for(nel * npe, 256, ctx->num_sms);
  k_n2e_count<<<g, 256, 0, s>>>(conn, emat, nel, npe, cnt);
  LLF_CUDA_TRY(ctx, dalloc(ctx, &ptr, non + 1));
  int64_t total = 0;
  LLF_CUDA_TRY(ctx, exclusive_scan_i64(ctx, cnt, ptr, non + 1, &total));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &list, total));
  LLF_CUDA_TRY(ctx, cudaMemsetAsync(cnt, 0, sizeof(int64_t) * (non + 1), s));
  k_n2e_fill<<<g, 256, 0, s>>>(conn, emat, nel, npe, ptr, cnt, list);
  int *d_max = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &d_max, 1));
  LLF_CUDA_TRY(ctx, cudaMemsetAsync(d_max, 0, sizeof(int), s));
  k_n2e_sort<<<grid_for(non, 128, ctx->num_sms), 128, 0, s>>>(ptr, list, non, d_max);
  int hmax = 0;
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(&hmax, d_max, sizeof(int), cudaMemcpyDeviceToHost, s));
  LLF_CUDA_TRY(ctx, cudaStreamSynchronize(s));
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  dfree(ctx, d_max);
  dfree(ctx, cnt);
  *ptr_out = ptr;
  *list_out = list;
  *max_len = hmax;
  return LLF_OK;
}

// Element-to-column map, one warp per column node: for every (element of
// the node's list, local node) pair, the row node's position in the column,
// by binary search in the sorted row-node list.
__global__ void k_row_positions(const int64_t *__restrict__ nptr, const int32_t *__restrict__ nadj,
                                const int64_t *__restrict__ n2e_ptr, const int2 *__restrict__ n2e,
                                const int32_t *__restrict__ conn, int npe, int64_t non,
                                uint16_t *__restrict__ pos, unsigned *status) {
  const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
  for (int64_t B = (int64_t)blockIdx.x * wpb + (threadIdx.x >> 5); B < non; B += (int64_t)gridDim.x * wpb) {
    const int64_t c0 = nptr[B];
    const int deg = (int)(nptr[B + 1] - c0);
    const int64_t s = n2e_ptr[B];
    const int64_t m = (n2e_ptr[B + 1] - s) * npe;
    for (int64_t it = lane; it < m; it += 32) {
      const int64_t k = it / npe;
      const int a = (int)(it - k * npe);
      const int A = conn[(size_t)n2e[s + k].x * npe + a];
      int lo = 0, hi = deg - 1;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (nadj[c0 + mid] < A) lo = mid + 1; else hi = mid;
      }
      uint16_t p = (uint16_t)lo;
      if (deg == 0 || nadj[c0 + lo] != A) {
        atomicOr(status, ST_PATTERN);
        p = 0xffff;
      }
      pos[s * npe + it] = p;
    }
  }
}

int row_positions(llf_ctx *ctx, const llf_pattern *pat, const int32_t *conn, int npe, const int64_t *n2e_ptr,
                  const int2 *n2e, int64_t n2e_total, uint16_t **pos) {
  *pos = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, pos, (size_t)n2e_total * npe));
  const int64_t non = pat->mesh->non;
  k_row_positions<<<grid_for(non * 32, 256, ctx->num_sms), 256, 0, ctx->stream>>>(
      pat->d_nptr, pat->d_nadj, n2e_ptr, n2e, conn, npe, non, *pos, ctx->d_status);
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  return LLF_OK;
}

int pattern_build_impl(llf_ctx *ctx, llf_mesh *mesh, int pdim, llf_pattern *pat) {
  const int64_t non = mesh->non, nel = mesh->nel;
  const int npe = mesh->npe;
  cudaStream_t s = ctx->stream;
  pat->mesh = mesh;
  pat->pdim = pdim;
  pat->ndof = non * pdim;

  // 1. node -> element lists
  int64_t *cnt = nullptr;
  int hmax = 0;
  int rc = build_n2e(ctx, mesh->d_conn, mesh->d_emat, nel, npe, non, &pat->d_n2e_ptr, &pat->d_n2e, &hmax);
  if (rc != LLF_OK) return rc;
  pat->max_n2e = hmax;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &cnt, non + 1));

  // 2. node adjacency (count, scan, fill)
  int64_t m = (int64_t)hmax * npe;
  int cap = 32;
  while (cap < m) cap <<= 1;
  const int warps = 4;
  size_t smem = (size_t)cap * warps * sizeof(int32_t);
  if (smem > 200 * 1024) {
    dfree(ctx, cnt);
    return llf_fail(ctx, LLF_ERR_LIMIT,
                    "pattern: a node's element neighbourhood holds " + std::to_string(m) +
                        " node slots; the limit is " + std::to_string(200 * 1024 / 16));
  }
  if (smem > 48 * 1024) {
    LLF_CUDA_TRY(ctx, cudaFuncSetAttribute(k_node_adjacency<false>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem));
    LLF_CUDA_TRY(ctx, cudaFuncSetAttribute(k_node_adjacency<true>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem));
  }
  unsigned gb = grid_for(non * 32, warps * 32, ctx->num_sms);
  LLF_CUDA_TRY(ctx, cudaMemsetAsync(cnt, 0, sizeof(int64_t) * (non + 1), s));
  k_node_adjacency<false><<<gb, warps * 32, smem, s>>>(mesh->d_conn, npe, pat->d_n2e_ptr,
                                                       pat->d_n2e, non, cap, cnt, nullptr,
                                                       nullptr, ctx->d_status);
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  {
    int *d_md = nullptr;
    LLF_CUDA_TRY(ctx, dalloc(ctx, &d_md, 1));
    LLF_CUDA_TRY(ctx, cudaMemsetAsync(d_md, 0, sizeof(int), s));
    k_max_deg<<<grid_for(non, 256, ctx->num_sms), 256, 0, s>>>(cnt, non, d_md);
    int md = 0;
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(&md, d_md, sizeof(int), cudaMemcpyDeviceToHost, s));
    LLF_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    dfree(ctx, d_md);
    pat->max_deg = md;
  }
  LLF_CUDA_TRY(ctx, dalloc(ctx, &pat->d_nptr, non + 1));
  int64_t nnzb = 0;
  LLF_CUDA_TRY(ctx, exclusive_scan_i64(ctx, cnt, pat->d_nptr, non + 1, &nnzb));
  pat->nnzb = nnzb;
  pat->nnz = nnzb * pdim * pdim;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &pat->d_nadj, nnzb));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &pat->d_diagpos, non));
  LLF_CUDA_TRY(ctx, cudaMemsetAsync(pat->d_diagpos, 0xff, sizeof(int32_t) * non, s));
  k_node_adjacency<true><<<gb, warps * 32, smem, s>>>(mesh->d_conn, npe, pat->d_n2e_ptr,
                                                      pat->d_n2e, non, cap, pat->d_nptr,
                                                      pat->d_nadj, pat->d_diagpos,
                                                      ctx->d_status);
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  dfree(ctx, cnt);

  // 3. DoF-level column pointers
  LLF_CUDA_TRY(ctx, dalloc(ctx, &pat->d_colptr, pat->ndof + 1));
  k_dof_colptr<<<grid_for(non, 256, ctx->num_sms), 256, 0, s>>>(pat->d_nptr, non, pdim,
                                                                pat->d_colptr);
  LLF_CUDA_TRY(ctx, cudaGetLastError());

  // 4. element-to-column map (positions fit 16 bits)
  if (pat->max_deg > 0xfffe)
    return llf_fail(ctx, LLF_ERR_LIMIT, "pattern: a column node has more than 65534 row nodes");
  int64_t n2e_total = 0;
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(&n2e_total, pat->d_n2e_ptr + non, sizeof(int64_t),
                                    cudaMemcpyDeviceToHost, s));
  LLF_CUDA_TRY(ctx, cudaStreamSynchronize(s));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &pat->d_pos, (size_t)n2e_total * npe));
  k_row_positions<<<grid_for(non * 32, 256, ctx->num_sms), 256, 0, s>>>(
      pat->d_nptr, pat->d_nadj, pat->d_n2e_ptr, pat->d_n2e, mesh->d_conn, npe, non, pat->d_pos,
      ctx->d_status);
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  pat->conn_version = mesh->conn_version;
  return llf_check_status(ctx, "llf_pattern_build");
}
