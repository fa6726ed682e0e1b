// fem_separate.cuh -- sparse separation of the assembled stiffness by the
// imposed displacements (included by fem_gpu.cu, whose handle and CSR it uses).
//
// methods_for_separate_stiffness_matrix.rs:217-320
// (separate_stiffness_matrix_sparse_iterative):
//   * diag[i] = K(i, i), 0 where the pattern has no diagonal entry;
//   * DOFs are taken in ascending order: diag 0 -> excluded, or an error if a
//     displacement is imposed on it (the first such DOF is reported);
//     otherwise restrained (b) when a displacement is imposed, else free (a);
//   * no restrained DOF -> "No restraints";
//   * every stored K(i, j) != 0 whose DOFs are both kept goes to K_aa, K_ab,
//     K_ba or K_bb with local indices (positions in the a and b lists);
//   * an empty K_aa -> the reference's "K_aa is empty" error.
// The reference collects the triplets in hash-map order; here every block is
// a CSR matrix sorted by (row, column) -- the same set of triplets.  Four
// lanes per stiffness row read it in order; each entry's position is the row's
// start plus the kept entries before it (ballot prefixes), so the result is
// deterministic.

enum : uint8_t { kSepExcluded = 0, kSepA = 1, kSepB = 2 };
constexpr int kSepBlocks = 4;  // K_aa, K_ab, K_ba, K_bb

// per DOF: its class (from the diagonal and the imposed displacements) and the first error
__global__ void k_sep_classify(size_t n, const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ col_idx,
                               const double* __restrict__ val, const uint8_t* __restrict__ imposed,
                               uint8_t* __restrict__ cls, uint32_t* __restrict__ isA, uint32_t* __restrict__ isB,
                               unsigned long long* __restrict__ first_err) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int64_t lo = row_ptr[i], hi = row_ptr[i + 1];
  const int64_t end = hi;
  while (lo < hi) {  // first entry with column >= i
    const int64_t mid = (lo + hi) >> 1;
    if (col_idx[mid] < (int32_t)i) lo = mid + 1;
    else hi = mid;
  }
  const double d = (lo < end && col_idx[lo] == (int32_t)i) ? val[lo] : 0.0;
  const bool con = imposed[i] != 0;
  uint8_t c;
  if (!nonzero(d)) {
    c = kSepExcluded;
    if (con) atomicMin(first_err, (unsigned long long)i);
  } else {
    c = con ? kSepB : kSepA;
  }
  cls[i] = c;
  isA[i] = c == kSepA;
  isB[i] = c == kSepB;
}

// Four lanes per stiffness row, eight rows per warp: a row of ~20 entries would leave most of a whole
// warp idle and make every warp a chain of dependent loads; with four lanes each load instruction reads
// four consecutive entries of eight rows.
constexpr int kSepLanes = 4;

// how many kept entries each row sends to each block; cnt is kSepBlocks x n, by global row
__global__ void k_sep_count(size_t n, const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ col_idx,
                            const double* __restrict__ val, const uint8_t* __restrict__ cls, uint32_t* __restrict__ cnt) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t row = t / kSepLanes;
  const int sub = (int)(t % kSepLanes);
  const uint8_t ci = row < n ? cls[row] : kSepExcluded;
  const int64_t b = row < n ? row_ptr[row] : 0;
  const int64_t e = ci != kSepExcluded ? row_ptr[row + 1] : b;
  uint32_t na = 0, nb = 0;
  for (int64_t k = b + sub; __any_sync(0xffffffffu, k < e); k += kSepLanes) {
    uint8_t cj = kSepExcluded;
    if (k < e && nonzero(val[k])) cj = cls[col_idx[k]];
    na += cj == kSepA;
    nb += cj == kSepB;
  }
#pragma unroll
  for (int o = 1; o < kSepLanes; o <<= 1) {
    na += __shfl_xor_sync(0xffffffffu, na, o);
    nb += __shfl_xor_sync(0xffffffffu, nb, o);
  }
  if (row < n && sub == 0) {
    cnt[0 * n + row] = ci == kSepA ? na : 0;  // K_aa
    cnt[1 * n + row] = ci == kSepA ? nb : 0;  // K_ab
    cnt[2 * n + row] = ci == kSepB ? na : 0;  // K_ba
    cnt[3 * n + row] = ci == kSepB ? nb : 0;  // K_bb
  }
}

// per DOF: its local index lists and the blocks' row pointers (rows of kept DOFs only)
__global__ void k_sep_rows(size_t n, const uint8_t* __restrict__ cls, const uint32_t* __restrict__ posA,
                           const uint32_t* __restrict__ posB, const unsigned long long* __restrict__ scan,
                           int64_t* __restrict__ a_idx, int64_t* __restrict__ b_idx, int64_t* __restrict__ rp_aa,
                           int64_t* __restrict__ rp_ab, int64_t* __restrict__ rp_ba, int64_t* __restrict__ rp_bb) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i > n) return;
  const size_t stride = n + 1;
  if (i == n) {  // totals close the row pointers
    rp_aa[posA[n]] = (int64_t)scan[0 * stride + n];
    rp_ab[posA[n]] = (int64_t)scan[1 * stride + n];
    rp_ba[posB[n]] = (int64_t)scan[2 * stride + n];
    rp_bb[posB[n]] = (int64_t)scan[3 * stride + n];
    return;
  }
  if (cls[i] == kSepA) {
    a_idx[posA[i]] = (int64_t)i;
    rp_aa[posA[i]] = (int64_t)scan[0 * stride + i];
    rp_ab[posA[i]] = (int64_t)scan[1 * stride + i];
  } else if (cls[i] == kSepB) {
    b_idx[posB[i]] = (int64_t)i;
    rp_ba[posB[i]] = (int64_t)scan[2 * stride + i];
    rp_bb[posB[i]] = (int64_t)scan[3 * stride + i];
  }
}

struct SepOut {
  int32_t* ci[kSepBlocks];
  double* v[kSepBlocks];
};

// every kept entry at its position (row start + the count of kept entries before it in the row, from the
// ballots of the row's four lanes), local column index
__global__ void k_sep_fill(size_t n, const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ col_idx,
                           const double* __restrict__ val, const uint8_t* __restrict__ cls,
                           const uint32_t* __restrict__ posA, const uint32_t* __restrict__ posB,
                           const unsigned long long* __restrict__ scan, SepOut out) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t row = t / kSepLanes;
  const int sub = (int)(t % kSepLanes);
  const int shift = (int)(threadIdx.x & 31) & ~(kSepLanes - 1);
  const uint8_t ci = row < n ? cls[row] : kSepExcluded;
  const int64_t b = row < n ? row_ptr[row] : 0;
  const int64_t e = ci != kSepExcluded ? row_ptr[row + 1] : b;
  const size_t stride = n + 1;
  const int ba = ci == kSepA ? 0 : 2;  // block of (row class, column a); +1 for column b
  unsigned long long pa = 0, pb = 0;
  if (ci != kSepExcluded) {
    pa = scan[(size_t)ba * stride + row];
    pb = scan[(size_t)(ba + 1) * stride + row];
  }
  const unsigned below = (1u << sub) - 1u, group = (1u << kSepLanes) - 1u;
  for (int64_t k0 = b; __any_sync(0xffffffffu, k0 < e); k0 += kSepLanes) {
    const int64_t k = k0 + sub;
    uint8_t cj = kSepExcluded;
    int32_t c = 0;
    double v = 0.0;
    if (k < e) {
      v = val[k];
      c = col_idx[k];
      if (nonzero(v)) cj = cls[c];
    }
    const unsigned ma = (__ballot_sync(0xffffffffu, cj == kSepA) >> shift) & group;
    const unsigned mb = (__ballot_sync(0xffffffffu, cj == kSepB) >> shift) & group;
    if (cj == kSepA) {
      const unsigned long long at = pa + __popc(ma & below);
      out.ci[ba][at] = (int32_t)posA[c];
      out.v[ba][at] = v;
    } else if (cj == kSepB) {
      const unsigned long long at = pb + __popc(mb & below);
      out.ci[ba + 1][at] = (int32_t)posB[c];
      out.v[ba + 1][at] = v;
    }
    pa += __popc(ma);
    pb += __popc(mb);
  }
}

namespace {
const char* const kDofNames[6] = {"X", "Y", "Z", "ThX", "ThY", "ThZ"};
}  // namespace

extern "C" int fem_gpu_separate_sparse(fem_gpu_t* h, const uint8_t* imposed) {
  if (!h || !imposed) return FEM_GPU_ERR_ARGUMENT;
  h->sep_valid = false;
  h->sell_valid = false;
  if (!h->pattern_valid || !h->numeric_done) return h->fail(FEM_GPU_ERR_STATE, "call fem_gpu_assemble first");
  cudaStream_t s = h->stream;
  const size_t n = (size_t)h->nodes_number * 6;
  CK(h->sep_imposed.reserve(n + 1, s));
  CK(h->sep_cls.reserve(n + 1, s));
  CK(h->sep_u32.reserve(4 * (n + 1) + kSepBlocks * n + 1, s));  // isA, isB, posA, posB, counts
  CK(h->sep_scan.reserve(kSepBlocks * (n + 1), s));
  CK(h->sep_err.reserve(1, s));
  uint32_t* isA = h->sep_u32.p;
  uint32_t* isB = isA + (n + 1);
  uint32_t* posA = isB + (n + 1);
  uint32_t* posB = posA + (n + 1);
  uint32_t* cnt = posB + (n + 1);
  if (n) CK(cudaMemcpyAsync(h->sep_imposed.p, imposed, n, cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(h->sep_err.p, 0xff, sizeof(unsigned long long), s));
  CK(cudaMemsetAsync(isA + n, 0, sizeof(uint32_t), s));
  CK(cudaMemsetAsync(isB + n, 0, sizeof(uint32_t), s));
  if (n) {
    k_sep_classify<<<grid_for(n, 256), 256, 0, s>>>(n, h->row_ptr.p, h->col_idx.p, h->values.p, h->sep_imposed.p,
                                                     h->sep_cls.p, isA, isB, h->sep_err.p);
    CK(cudaGetLastError());
  }
  unsigned long long first_err = 0;
  CK(cudaMemcpyAsync(&first_err, h->sep_err.p, sizeof first_err, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (first_err != ~0ull) {
    const size_t node = (size_t)(first_err / 6);
    const uint32_t number = node < h->n_nodes ? h->idx_number[node] : 0u;
    return h->fail(FEM_GPU_ERR_SEP_DISPLACEMENT,
                   "There are no stiffness to withstand displacement %s applied to node %u!",
                   kDofNames[first_err % 6], number);
  }
  // local positions: exclusive scans over n + 1 entries (the last one is the count)
  int st = cub_call(h, [&](void* tmp, size_t& bytes) {
    return cub::DeviceScan::ExclusiveSum(tmp, bytes, isA, posA, (int64_t)(n + 1), s);
  });
  if (st) return st;
  st = cub_call(h, [&](void* tmp, size_t& bytes) {
    return cub::DeviceScan::ExclusiveSum(tmp, bytes, isB, posB, (int64_t)(n + 1), s);
  });
  if (st) return st;
  uint32_t nab[2] = {0, 0};
  CK(cudaMemcpyAsync(&nab[0], posA + n, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(&nab[1], posB + n, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  h->sep_n[0] = nab[0];
  h->sep_n[1] = nab[1];
  if (nab[1] == 0) return h->fail(FEM_GPU_ERR_SEP_NO_RESTRAINTS, "No restraints");
  // per-row counts of each block, their scans (n + 1 each: the last entry is the block's size)
  if (n) {
    k_sep_count<<<grid_for(n * kSepLanes, 256), 256, 0, s>>>(n, h->row_ptr.p, h->col_idx.p, h->values.p,
                                                              h->sep_cls.p, cnt);
    CK(cudaGetLastError());
  }
  for (int b = 0; b < kSepBlocks; ++b) {
    CK(cudaMemsetAsync(h->sep_scan.p + (size_t)b * (n + 1) + n, 0, sizeof(unsigned long long), s));
    if (!n) continue;
    unsigned long long* out = h->sep_scan.p + (size_t)b * (n + 1);
    const uint32_t* in = cnt + (size_t)b * n;
    // inclusive scan written one place on: out[0] = 0, out[i + 1] = sum of the first i + 1 counts
    CK(cudaMemsetAsync(out, 0, sizeof(unsigned long long), s));
    st = cub_call(h, [&](void* tmp, size_t& bytes) {
      return cub::DeviceScan::InclusiveSum(tmp, bytes, in, out + 1, (int64_t)n, s);
    });
    if (st) return st;
  }
  unsigned long long tot[kSepBlocks];
  for (int b = 0; b < kSepBlocks; ++b)
    CK(cudaMemcpyAsync(&tot[b], h->sep_scan.p + (size_t)b * (n + 1) + n, sizeof(unsigned long long),
                       cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  for (int b = 0; b < kSepBlocks; ++b) h->sep_nnz[b] = (int64_t)tot[b];
  if (tot[0] == 0)
    return h->fail(FEM_GPU_ERR_SEP_EMPTY_KAA, "Sparse separation: K_aa is empty (structure has no free stiffness?)");
  // index lists, row pointers, entries
  CK(h->sep_idx.reserve((size_t)nab[0] + nab[1] + 1, s));
  const size_t rows[kSepBlocks] = {nab[0], nab[0], nab[1], nab[1]};
  for (int b = 0; b < kSepBlocks; ++b) {
    CK(h->sep_rp[b].reserve(rows[b] + 1, s));
    CK(h->sep_ci[b].reserve((size_t)tot[b] + 1, s));
    CK(h->sep_v[b].reserve((size_t)tot[b] + 1, s));
  }
  k_sep_rows<<<grid_for(n + 1, 256), 256, 0, s>>>(n, h->sep_cls.p, posA, posB, h->sep_scan.p, h->sep_idx.p,
                                                   h->sep_idx.p + nab[0], h->sep_rp[0].p, h->sep_rp[1].p,
                                                   h->sep_rp[2].p, h->sep_rp[3].p);
  SepOut o;
  for (int b = 0; b < kSepBlocks; ++b) {
    o.ci[b] = h->sep_ci[b].p;
    o.v[b] = h->sep_v[b].p;
  }
  if (n)
    k_sep_fill<<<grid_for(n * kSepLanes, 256), 256, 0, s>>>(n, h->row_ptr.p, h->col_idx.p, h->values.p,
                                                             h->sep_cls.p, posA, posB, h->sep_scan.p, o);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(s));
  h->sep_valid = true;
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_get_separation_sizes(fem_gpu_t* h, int64_t* n_aa, int64_t* n_bb, int64_t* nnz4) {
  if (!h) return FEM_GPU_ERR_ARGUMENT;
  if (!h->sep_valid) return h->fail(FEM_GPU_ERR_STATE, "call fem_gpu_separate_sparse first");
  if (n_aa) *n_aa = h->sep_n[0];
  if (n_bb) *n_bb = h->sep_n[1];
  if (nnz4)
    for (int b = 0; b < kSepBlocks; ++b) nnz4[b] = h->sep_nnz[b];
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_get_separation_indexes(fem_gpu_t* h, int64_t* aa_indexes, int64_t* bb_indexes) {
  if (!h) return FEM_GPU_ERR_ARGUMENT;
  if (!h->sep_valid) return h->fail(FEM_GPU_ERR_STATE, "call fem_gpu_separate_sparse first");
  if (aa_indexes && h->sep_n[0])
    CK(cudaMemcpyAsync(aa_indexes, h->sep_idx.p, h->sep_n[0] * 8, cudaMemcpyDeviceToHost, h->stream));
  if (bb_indexes && h->sep_n[1])
    CK(cudaMemcpyAsync(bb_indexes, h->sep_idx.p + h->sep_n[0], h->sep_n[1] * 8, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_get_separation_block(fem_gpu_t* h, int which, int64_t* row_ptr, int32_t* col_idx,
                                            double* values) {
  if (!h || which < 0 || which >= kSepBlocks) return FEM_GPU_ERR_ARGUMENT;
  if (!h->sep_valid) return h->fail(FEM_GPU_ERR_STATE, "call fem_gpu_separate_sparse first");
  const size_t rows = which < 2 ? (size_t)h->sep_n[0] : (size_t)h->sep_n[1];
  const size_t nz = (size_t)h->sep_nnz[which];
  if (row_ptr) CK(cudaMemcpyAsync(row_ptr, h->sep_rp[which].p, (rows + 1) * 8, cudaMemcpyDeviceToHost, h->stream));
  if (col_idx && nz) CK(cudaMemcpyAsync(col_idx, h->sep_ci[which].p, nz * 4, cudaMemcpyDeviceToHost, h->stream));
  if (values && nz) CK(cudaMemcpyAsync(values, h->sep_v[which].p, nz * 8, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_get_separation_block_device(fem_gpu_t* h, int which, const int64_t** row_ptr,
                                                   const int32_t** col_idx, const double** values) {
  if (!h || which < 0 || which >= kSepBlocks) return FEM_GPU_ERR_ARGUMENT;
  if (!h->sep_valid) return h->fail(FEM_GPU_ERR_STATE, "call fem_gpu_separate_sparse first");
  if (row_ptr) *row_ptr = h->sep_rp[which].p;
  if (col_idx) *col_idx = h->sep_ci[which].p;
  if (values) *values = h->sep_v[which].p;
  return FEM_GPU_OK;
}
