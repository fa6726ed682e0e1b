// fem_solve.cuh -- iterative solution of the separated system and the
// reactions (included by fem_gpu.cu after fem_separate.cuh).
//
// methods_for_global_analysis.rs:189-275 and :100-133:
//   b   = r_a - K_ab u_b                     (find_b_sparse)
//   u_a : K_aa u_a = b by preconditioned conjugate gradients from u_a = 0, the
//         preconditioner the diagonal of K_aa (pcg_jacobi_csr) or its node blocks
//         (pcg_block_jacobi_csr, blocks = the free DOFs of one node,
//         build_block_starts_from_k_aa_indexes)
//   r_r = K_ba u_a + K_bb u_b - r_b          (find_r_r_sparse)
// The PCG itself lives in the unvendored iterative_solvers_smpl 0.1.5; this is
// the textbook recurrence with the stopping rule ||r||_2 <= max(rel_tol ||b||_2,
// abs_tol), checked after every iteration.  Every sum runs in a fixed order
// (fixed grids, fixed reduction trees), so results repeat run to run.

// The conjugate-gradient loop runs on K_aa in a sliced ELLPACK copy (SELL-C-sigma: slices of 32 rows stored
// column-major, rows sorted by length inside windows of 1024 rows so a slice's rows have nearly equal lengths):
// one thread per row, 32 consecutive rows read coalesced, one FMA per stored entry and no reduction tree.  On this
// GPU the CSR product sits at the ridge of FP64 rate and HBM bandwidth (one FMA per 12 bytes), so the lanes-per-row
// partial sums and their shuffle adds cost as much as the matrix traffic; the slices remove them.  The copy is
// built once per separation.  Dot products are fused into the kernels that produce their operands (block
// partials in a fixed order, then one block sums the partials and updates the recurrence's scalars on the
// device), and the stopping test runs on the device too: the host enqueues iterations in growing batches and
// reads the state once per batch; kernels of iterations past convergence return at once.

// y[i] = sum_j K[i][j] x[j], or a (s[i] - that sum) when s is given (CSR, kLanesPerRow lanes per row): the
// one-off products b = r_a - K_ab u_b and the reactions
constexpr int kLanesPerRow = 4;
__global__ void k_spmv(size_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                       const double* __restrict__ v, const double* __restrict__ x, const double* __restrict__ s,
                       double a, double* __restrict__ y) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t row = t / kLanesPerRow;
  const int sub = (int)(t % kLanesPerRow);
  double acc = 0.0;
  if (row < n)
    for (int64_t k = rp[row] + sub; k < rp[row + 1]; k += kLanesPerRow) acc = fma(v[k], x[ci[k]], acc);
#pragma unroll
  for (int o = kLanesPerRow / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (row < n && sub == 0) y[row] = s ? a * (s[row] - acc) : acc;
}

// y[i] = y[i] + sum_j K[i][j] x[j] (row-wise), used for the reactions
__global__ void k_spmv_add(size_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                           const double* __restrict__ v, const double* __restrict__ x, double* __restrict__ y) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t row = t / kLanesPerRow;
  const int sub = (int)(t % kLanesPerRow);
  double acc = 0.0;
  if (row < n)
    for (int64_t k = rp[row] + sub; k < rp[row + 1]; k += kLanesPerRow) acc = fma(v[k], x[ci[k]], acc);
#pragma unroll
  for (int o = kLanesPerRow / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (row < n && sub == 0) y[row] = y[row] + acc;
}

constexpr int kSellC = 32;                          // rows per slice
constexpr int kSellThreads = 256;                   // one window per CTA
constexpr int kSellSlicesPerWarp = 4;
constexpr int kSellWindow = kSellThreads / 32 * kSellSlicesPerWarp * kSellC;  // 1024 rows
constexpr int kSellSortItems = kSellWindow / kSellThreads;                    // 4 rows per thread in the sort
constexpr uint32_t kNoRow = 0xffffffffu;
constexpr int kVecThreads = 256, kVecBlocks = 1184;  // grid-stride vector kernels: 8 CTAs per SM
constexpr uint32_t kInfoStartMask = (1u << 29) - 1u;  // per DOF: its preconditioner block's start | size << 29

// sum of v over the CTA in a fixed order (warp xor tree, then warp partials in order); valid in thread 0
template <int kThreads>
__device__ __forceinline__ double cta_sum(double v, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < kThreads / 32; ++k) t += sh[k];
  return t;
}

// --- sliced ELLPACK copy of K_aa -----------------------------------------------------------------------------
// per window: its rows sorted by length (descending, stable), the permutation, and each slice's width
__global__ void __launch_bounds__(kSellThreads) k_sell_sort(size_t n, const int64_t* __restrict__ rp,
                                                            uint32_t* __restrict__ perm, int64_t* __restrict__ width) {
  using Sort = cub::BlockRadixSort<uint32_t, kSellThreads, kSellSortItems, uint32_t>;
  __shared__ typename Sort::TempStorage tmp;
  uint32_t key[kSellSortItems], val[kSellSortItems];
  const size_t base = (size_t)blockIdx.x * kSellWindow;
#pragma unroll
  for (int k = 0; k < kSellSortItems; ++k) {
    const size_t row = base + (size_t)threadIdx.x * kSellSortItems + k;
    key[k] = row < n ? (uint32_t)(rp[row + 1] - rp[row]) : 0u;
    val[k] = row < n ? (uint32_t)row : kNoRow;
  }
  Sort(tmp).SortDescending(key, val);
#pragma unroll
  for (int k = 0; k < kSellSortItems; ++k) perm[base + (size_t)threadIdx.x * kSellSortItems + k] = val[k];
  // the first row of every slice is its longest: slice j starts at item 32 j, held by thread 8 j
  if ((threadIdx.x * kSellSortItems) % kSellC == 0)
    width[(size_t)blockIdx.x * (kSellWindow / kSellC) + threadIdx.x * kSellSortItems / kSellC] =
        (int64_t)kSellC * key[0];
}

// the slices, column-major (entry k of the slice's lane l at off + 32 k + l); rows shorter than their slice are
// padded with zeros at their own first column
__global__ void k_sell_fill(size_t n_pos, const uint32_t* __restrict__ perm, const int64_t* __restrict__ off,
                            const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                            const double* __restrict__ v, int32_t* __restrict__ col, double* __restrict__ val) {
  const size_t pos = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (pos >= n_pos) return;
  const size_t sl = pos / kSellC;
  const int lane = (int)(pos % kSellC);
  const int64_t o = off[sl], w = (off[sl + 1] - o) / kSellC;
  const uint32_t row = perm[pos];
  const int64_t b = row != kNoRow ? rp[row] : 0, len = row != kNoRow ? rp[row + 1] - b : 0;
  const int32_t pad = row != kNoRow ? ci[b] : 0;
  for (int64_t k = 0; k < w; ++k) {
    const int64_t at = o + kSellC * k + lane;
    col[at] = k < len ? ci[b + k] : pad;
    val[at] = k < len ? v[b + k] : 0.0;
  }
}

// q = K p and the CTA's partial of p . q; a warp takes four slices
__global__ void __launch_bounds__(kSellThreads) k_sell_spmv_dot(size_t n_windows, const int64_t* __restrict__ off,
                                                                const uint32_t* __restrict__ perm,
                                                                const int32_t* __restrict__ col,
                                                                const double* __restrict__ val,
                                                                const double* __restrict__ p, double* __restrict__ q,
                                                                double* __restrict__ part, const int* __restrict__ state) {
  __shared__ double sh[kSellThreads / 32];
  if (*state) return;
  const int lane = threadIdx.x & 31;
  const size_t warp = (size_t)blockIdx.x * (kSellThreads / 32) + (threadIdx.x >> 5);
  double dot = 0.0;
  if (blockIdx.x < n_windows) {
#pragma unroll 1
    for (int j = 0; j < kSellSlicesPerWarp; ++j) {
      const size_t sl = warp * kSellSlicesPerWarp + j;
      const int64_t o = off[sl], w = (off[sl + 1] - o) / kSellC;
      const double* vv = val + o + lane;
      const int32_t* cc = col + o + lane;
      double acc = 0.0;
      int64_t k = 0;
      // four entries per step: their loads and gathers are issued before the first FMA needs one (the sum
      // still runs entry by entry)
      for (; k + 4 <= w; k += 4) {
        const int32_t c0 = __ldg(cc + kSellC * k), c1 = __ldg(cc + kSellC * (k + 1)),
                      c2 = __ldg(cc + kSellC * (k + 2)), c3 = __ldg(cc + kSellC * (k + 3));
        const double v0 = __ldg(vv + kSellC * k), v1 = __ldg(vv + kSellC * (k + 1)),
                     v2 = __ldg(vv + kSellC * (k + 2)), v3 = __ldg(vv + kSellC * (k + 3));
        const double x0 = __ldg(p + c0), x1 = __ldg(p + c1), x2 = __ldg(p + c2), x3 = __ldg(p + c3);
        acc = fma(v0, x0, acc);
        acc = fma(v1, x1, acc);
        acc = fma(v2, x2, acc);
        acc = fma(v3, x3, acc);
      }
      for (; k < w; ++k) acc = fma(__ldg(vv + kSellC * k), __ldg(p + __ldg(cc + kSellC * k)), acc);
      const uint32_t row = perm[sl * kSellC + lane];
      if (row != kNoRow) {
        q[row] = acc;
        dot = fma(p[row], acc, dot);
      }
    }
  }
  const double t = cta_sum<kSellThreads>(dot, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// --- preconditioner ------------------------------------------------------------------------------------------
// blocks: the free DOFs of one node (consecutive in the a list); start of each block per DOF
__global__ void k_block_heads(size_t n, const int64_t* __restrict__ a_idx, uint32_t* __restrict__ head) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  head[i] = (i == 0 || a_idx[i] / 6 != a_idx[i - 1] / 6) ? 1u : 0u;
}

// start of each block: the DOFs with a head flag, at their rank among the heads
__global__ void k_block_starts_of(size_t n, const uint32_t* __restrict__ head, const uint32_t* __restrict__ pos,
                                  uint32_t* __restrict__ start) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n && head[i]) start[pos[i]] = (uint32_t)i;
}

// the inverse of each diagonal block of K_aa (size <= 6) by Gauss-Jordan elimination with partial pivoting;
// blocks of size 1 are the Jacobi preconditioner.  Written per DOF: its row of the block's inverse (6 doubles,
// zero past the block's size) and its block's start and size
__global__ void k_block_inverse(size_t nblk, const uint32_t* __restrict__ start, size_t n,
                                const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                const double* __restrict__ v, double* __restrict__ inv_row,
                                uint32_t* __restrict__ info, int* singular) {
  const size_t b = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (b >= nblk) return;
  const uint32_t s = start[b], e = b + 1 < nblk ? start[b + 1] : (uint32_t)n;
  const int m = (int)(e - s);
  double A[36], X[36];
  for (int i = 0; i < 36; ++i) {
    A[i] = 0.0;
    X[i] = (i % 7 == 0) ? 1.0 : 0.0;
  }
  for (int i = 0; i < m; ++i)
    for (int64_t k = rp[s + i]; k < rp[s + i + 1]; ++k) {
      const int64_t c = ci[k];
      if (c >= (int64_t)s && c < (int64_t)e) A[6 * i + (int)(c - s)] = v[k];
    }
  for (int col = 0; col < m; ++col) {
    int piv = col;
    for (int r = col + 1; r < m; ++r)
      if (fabs(A[6 * r + col]) > fabs(A[6 * piv + col])) piv = r;
    if (A[6 * piv + col] == 0.0) {
      atomicOr(singular, 1);
      return;
    }
    if (piv != col)
      for (int k = 0; k < 6; ++k) {
        double t = A[6 * col + k];
        A[6 * col + k] = A[6 * piv + k];
        A[6 * piv + k] = t;
        t = X[6 * col + k];
        X[6 * col + k] = X[6 * piv + k];
        X[6 * piv + k] = t;
      }
    const double d = 1.0 / A[6 * col + col];
    for (int k = 0; k < 6; ++k) {
      A[6 * col + k] *= d;
      X[6 * col + k] *= d;
    }
    for (int r = 0; r < m; ++r) {
      if (r == col) continue;
      const double f = A[6 * r + col];
      if (f == 0.0) continue;
      for (int k = 0; k < 6; ++k) {
        A[6 * r + k] = fma(-f, A[6 * col + k], A[6 * r + k]);
        X[6 * r + k] = fma(-f, X[6 * col + k], X[6 * r + k]);
      }
    }
  }
  for (int i = 0; i < m; ++i) {
    for (int k = 0; k < 6; ++k) inv_row[6 * (size_t)(s + i) + k] = X[6 * i + k];
    info[s + i] = s | ((uint32_t)m << 29);
  }
}

// z = M^-1 r, one DOF per step, and the CTA's partial of r . z
__global__ void __launch_bounds__(kVecThreads) k_block_apply_dot(size_t n, const uint32_t* __restrict__ info,
                                                                 const double* __restrict__ inv_row,
                                                                 const double* __restrict__ r,
                                                                 double* __restrict__ z, double* __restrict__ part,
                                                                 const int* __restrict__ state) {
  __shared__ double sh[kVecThreads / 32];
  if (state && *state) return;
  double dot = 0.0;
  // two DOFs per step (i and i + stride), so each thread has two rows' loads in flight; the dot product still
  // adds the DOFs in the order i, i + stride, i + 2 stride, ...
  const size_t stride = (size_t)gridDim.x * kVecThreads;
  for (size_t i = blockIdx.x * (size_t)kVecThreads + threadIdx.x; i < n; i += 2 * stride) {
    const size_t i2 = i + stride;
    const bool two = i2 < n;
    const uint32_t in = info[i], in2 = two ? info[i2] : 0u;
    const double2* ir = reinterpret_cast<const double2*>(inv_row + 6 * i);
    const double2* ir2 = reinterpret_cast<const double2*>(inv_row + 6 * (two ? i2 : i));
    const double2 a = ir[0], b = ir[1], c = ir[2];
    const double2 a2 = ir2[0], b2 = ir2[1], c2 = ir2[2];
    const double w[6] = {a.x, a.y, b.x, b.y, c.x, c.y}, w2[6] = {a2.x, a2.y, b2.x, b2.y, c2.x, c2.y};
    const uint32_t s = in & kInfoStartMask, s2 = in2 & kInfoStartMask;
    const int m = (int)(in >> 29), m2 = (int)(in2 >> 29);
    double rs[6], rs2[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      rs[j] = j < m ? r[s + j] : 0.0;
      rs2[j] = j < m2 ? r[s2 + j] : 0.0;
    }
    const double ri = r[i], ri2 = two ? r[i2] : 0.0;
    double acc = 0.0, acc2 = 0.0;
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      if (j < m) acc = fma(w[j], rs[j], acc);
      if (j < m2) acc2 = fma(w2[j], rs2[j], acc2);
    }
    z[i] = acc;
    dot = fma(ri, acc, dot);
    if (two) {
      z[i2] = acc2;
      dot = fma(ri2, acc2, dot);
    }
  }
  const double t = cta_sum<kVecThreads>(dot, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// --- recurrence --------------------------------------------------------------------------------------------
// device scalars: r.z, p.Aq, r.r, alpha, beta, tolerance; state[0]: 0 running, 1 converged, 2 p.Aq <= 0 (the
// matrix is not positive definite); state[1]: iterations completed
enum { kRz = 0, kPq = 1, kRr = 2, kAlpha = 3, kBeta = 4, kTol = 5, kScalars = 6 };

// x . y partials over a fixed grid
__global__ void __launch_bounds__(kVecThreads) k_dot_part(size_t n, const double* __restrict__ x,
                                                          const double* __restrict__ y, double* __restrict__ part) {
  __shared__ double sh[kVecThreads / 32];
  double dot = 0.0;
  for (size_t i = blockIdx.x * (size_t)kVecThreads + threadIdx.x; i < n; i += (size_t)gridDim.x * kVecThreads)
    dot = fma(x[i], y[i], dot);
  const double t = cta_sum<kVecThreads>(dot, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// x += alpha p, r -= alpha q, and the CTA's partial of r . r
__global__ void __launch_bounds__(kVecThreads) k_cg_update_dot(size_t n, const double* __restrict__ sc,
                                                               const double* __restrict__ p,
                                                               const double* __restrict__ q, double* __restrict__ x,
                                                               double* __restrict__ r, double* __restrict__ part,
                                                               const int* __restrict__ state) {
  __shared__ double sh[kVecThreads / 32];
  if (*state) return;
  const double alpha = sc[kAlpha];
  double dot = 0.0;
  for (size_t i = blockIdx.x * (size_t)kVecThreads + threadIdx.x; i < n; i += (size_t)gridDim.x * kVecThreads) {
    x[i] = fma(alpha, p[i], x[i]);
    const double ri = fma(-alpha, q[i], r[i]);
    r[i] = ri;
    dot = fma(ri, ri, dot);
  }
  const double t = cta_sum<kVecThreads>(dot, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// p = z + beta p
__global__ void __launch_bounds__(kVecThreads) k_cg_direction(size_t n, const double* __restrict__ sc,
                                                              const double* __restrict__ z, double* __restrict__ p,
                                                              const int* __restrict__ state) {
  if (*state) return;
  const double beta = sc[kBeta];
  for (size_t i = blockIdx.x * (size_t)kVecThreads + threadIdx.x; i < n; i += (size_t)gridDim.x * kVecThreads)
    p[i] = fma(beta, p[i], z[i]);
}

// the partials' sum (fixed order), then the scalar step `op`:
//   0 start:  r.r of b; tolerance max(rel_tol |b|, abs_tol); converged already when |b| <= tolerance
//   1 r.z of the first preconditioned residual
//   2 alpha:  p.Aq; alpha = r.z / p.Aq (state 2 when p.Aq <= 0)
//   3 residual: r.r; one more iteration done; converged when |r| <= tolerance
//   4 beta:   r.z new; beta = r.z new / r.z; r.z = r.z new
constexpr int kFinalThreads = 256;
__global__ void __launch_bounds__(kFinalThreads) k_cg_scalar(int n_part, const double* __restrict__ part,
                                                             double* __restrict__ sc, int* __restrict__ state, int op,
                                                             double rel_tol, double abs_tol) {
  __shared__ double sh[kFinalThreads / 32];
  if (op != 0 && state[0]) return;
  double acc = 0.0;
  for (int i = threadIdx.x; i < n_part; i += kFinalThreads) acc += part[i];
  const double v = cta_sum<kFinalThreads>(acc, sh);
  if (threadIdx.x != 0) return;
  switch (op) {
    case 0: {
      sc[kRr] = v;
      const double tol = fmax(rel_tol * sqrt(v), abs_tol);
      sc[kTol] = tol;
      state[1] = 0;
      state[0] = !(sqrt(v) > tol) ? 1 : 0;
      break;
    }
    case 1:
      sc[kRz] = v;
      break;
    case 2:
      sc[kPq] = v;
      if (!(v > 0.0)) state[0] = 2;
      sc[kAlpha] = sc[kRz] / v;
      break;
    case 3:
      sc[kRr] = v;
      state[1] += 1;
      if (!(sqrt(v) > sc[kTol])) state[0] = 1;
      break;
    default:
      sc[kBeta] = v / sc[kRz];
      sc[kRz] = v;
      break;
  }
}

namespace {

// the sliced copy of K_aa, built once per separation
int sell_build(fem_gpu* h) {
  if (h->sell_valid) return FEM_GPU_OK;
  cudaStream_t s = h->stream;
  const size_t n = (size_t)h->sep_n[0];
  const size_t n_windows = (n + kSellWindow - 1) / kSellWindow;
  const size_t n_slices = n_windows * (kSellWindow / kSellC), n_pos = n_windows * kSellWindow;
  CK(h->sell_perm.reserve(n_pos + 1, s));
  CK(h->sell_off.reserve(n_slices + 1, s));
  DevBuf<int64_t> width;  // entries per slice (32 x its longest row), then 0
  CK(width.reserve(n_slices + 1, s));
  CK(cudaMemsetAsync(width.p + n_slices, 0, sizeof(int64_t), s));
  if (n_windows) k_sell_sort<<<(unsigned)n_windows, kSellThreads, 0, s>>>(n, h->sep_rp[0].p, h->sell_perm.p, width.p);
  CK(cudaGetLastError());
  int st = cub_call(h, [&](void* tmp, size_t& bytes) {
    return cub::DeviceScan::ExclusiveSum(tmp, bytes, width.p, h->sell_off.p, (int64_t)(n_slices + 1), s);
  });
  if (st) return st;
  int64_t total = 0;
  CK(cudaMemcpyAsync(&total, h->sell_off.p + n_slices, sizeof total, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  CK(h->sell_col.reserve((size_t)total + 1, s));
  CK(h->sell_val.reserve((size_t)total + 1, s));
  if (n_pos)
    k_sell_fill<<<grid_for(n_pos, 256), 256, 0, s>>>(n_pos, h->sell_perm.p, h->sell_off.p, h->sep_rp[0].p,
                                                     h->sep_ci[0].p, h->sep_v[0].p, h->sell_col.p, h->sell_val.p);
  CK(cudaGetLastError());
  h->sell_windows = n_windows;
  h->sell_entries = total;
  h->sell_valid = true;
  return FEM_GPU_OK;
}

unsigned vec_blocks(size_t n) {
  return (unsigned)std::max<size_t>(1, std::min<size_t>(kVecBlocks, (n + kVecThreads - 1) / kVecThreads));
}

}  // namespace

extern "C" int fem_gpu_solve_pcg(fem_gpu_t* h, const double* r_a, const double* u_b, int block_jacobi, int max_iter,
                                 double* u_a, int* iterations) {
  if (!h || !r_a || !u_a || max_iter < 0) return FEM_GPU_ERR_ARGUMENT;
  if (!h->sep_valid) return h->fail(FEM_GPU_ERR_STATE, "call fem_gpu_separate_sparse first");
  cudaStream_t s = h->stream;
  const size_t n = (size_t)h->sep_n[0], nbb = (size_t)h->sep_n[1];
  if (n > (size_t)kInfoStartMask) return h->fail(FEM_GPU_ERR_ARGUMENT, "too many free DOFs for the PCG (%zu)", n);
  if (iterations) *iterations = 0;
  int st = sell_build(h);
  if (st) return st;
  const size_t n_part = std::max<size_t>(kVecBlocks, h->sell_windows) + 1;
  CK(h->pcg_vec.reserve(6 * n + nbb + 1, s));
  CK(h->pcg_part.reserve(n_part, s));
  CK(h->pcg_scal.reserve(kScalars, s));
  CK(h->pcg_state.reserve(2, s));
  double* x = h->pcg_vec.p;
  double* r = x + n;
  double* z = r + n;
  double* p = z + n;
  double* q = p + n;
  double* ra = q + n;
  double* ub = ra + n;
  double* part = h->pcg_part.p;
  double* sc = h->pcg_scal.p;
  int* state = h->pcg_state.p;
  CK(cudaMemcpyAsync(ra, r_a, n * sizeof(double), cudaMemcpyHostToDevice, s));
  if (nbb) {
    if (u_b) CK(cudaMemcpyAsync(ub, u_b, nbb * sizeof(double), cudaMemcpyHostToDevice, s));
    else CK(cudaMemsetAsync(ub, 0, nbb * sizeof(double), s));
  }
  // b = r_a - K_ab u_b, kept in r (x = 0 so the first residual is b)
  if (n) {
    k_spmv<<<grid_for(n * kLanesPerRow, 256), 256, 0, s>>>(n, h->sep_rp[1].p, h->sep_ci[1].p, h->sep_v[1].p, ub, ra,
                                                            1.0, r);
    CK(cudaMemsetAsync(x, 0, n * sizeof(double), s));
  }
  // preconditioner: node blocks of the a list (block Jacobi) or single DOFs (Jacobi)
  size_t nblk = n;
  CK(h->pcg_blk.reserve(n + 1, s));
  if (block_jacobi && n) {
    DevBuf<uint32_t> head, pos;
    CK(head.reserve(n + 1, s));
    CK(pos.reserve(n + 1, s));
    CK(cudaMemsetAsync(head.p + n, 0, sizeof(uint32_t), s));
    k_block_heads<<<grid_for(n, 256), 256, 0, s>>>(n, h->sep_idx.p, head.p);
    st = cub_call(h, [&](void* tmp, size_t& bytes) {
      return cub::DeviceScan::ExclusiveSum(tmp, bytes, head.p, pos.p, (int64_t)(n + 1), s);
    });
    if (st) return st;
    k_block_starts_of<<<grid_for(n, 256), 256, 0, s>>>(n, head.p, pos.p, h->pcg_blk.p);
    uint32_t nb_host = 0;
    CK(cudaMemcpyAsync(&nb_host, pos.p + n, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    nblk = (size_t)nb_host;
  } else if (n) {
    k_iota<<<grid_for(n, 256), 256, 0, s>>>(n, h->pcg_blk.p);
  }
  CK(h->pcg_inv.reserve(6 * n + 1, s));
  CK(h->pcg_info.reserve(n + 1, s));
  CK(h->flag.reserve(1, s));
  CK(cudaMemsetAsync(h->flag.p, 0, sizeof(int), s));
  if (nblk)
    k_block_inverse<<<grid_for(nblk, 128), 128, 0, s>>>(nblk, h->pcg_blk.p, n, h->sep_rp[0].p, h->sep_ci[0].p,
                                                        h->sep_v[0].p, h->pcg_inv.p, h->pcg_info.p, h->flag.p);
  CK(cudaGetLastError());
  int singular = 0;
  CK(cudaMemcpyAsync(&singular, h->flag.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (singular) return h->fail(FEM_GPU_ERR_NOT_CONVERGED, "find_ua_vector_iterative: PCG failed: singular preconditioner");
  const unsigned vb = vec_blocks(n);
  const unsigned nw = (unsigned)std::max<size_t>(1, h->sell_windows);
  // start: |b|, the tolerance, z = M^-1 r, r.z, p = z
  k_dot_part<<<vb, kVecThreads, 0, s>>>(n, r, r, part);
  k_cg_scalar<<<1, kFinalThreads, 0, s>>>((int)vb, part, sc, state, 0, h->rel_tol, h->abs_tol);
  k_block_apply_dot<<<vb, kVecThreads, 0, s>>>(n, h->pcg_info.p, h->pcg_inv.p, r, z, part, state);
  k_cg_scalar<<<1, kFinalThreads, 0, s>>>((int)vb, part, sc, state, 1, 0.0, 0.0);
  CK(cudaMemcpyAsync(p, z, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  CK(cudaGetLastError());
  // iterations in batches of 1, 2, 4, ... 32 between reads of the state
  int host_state[2] = {0, 0};
  CK(cudaMemcpyAsync(host_state, state, sizeof host_state, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  int enqueued = 0, batch = 1;
  while (host_state[0] == 0 && enqueued < max_iter) {
    const int k = std::min(batch, max_iter - enqueued);
    for (int j = 0; j < k; ++j) {
      k_sell_spmv_dot<<<nw, kSellThreads, 0, s>>>(h->sell_windows, h->sell_off.p, h->sell_perm.p, h->sell_col.p,
                                                   h->sell_val.p, p, q, part, state);
      k_cg_scalar<<<1, kFinalThreads, 0, s>>>((int)nw, part, sc, state, 2, 0.0, 0.0);
      k_cg_update_dot<<<vb, kVecThreads, 0, s>>>(n, sc, p, q, x, r, part, state);
      k_cg_scalar<<<1, kFinalThreads, 0, s>>>((int)vb, part, sc, state, 3, 0.0, 0.0);
      k_block_apply_dot<<<vb, kVecThreads, 0, s>>>(n, h->pcg_info.p, h->pcg_inv.p, r, z, part, state);
      k_cg_scalar<<<1, kFinalThreads, 0, s>>>((int)vb, part, sc, state, 4, 0.0, 0.0);
      k_cg_direction<<<vb, kVecThreads, 0, s>>>(n, sc, z, p, state);
    }
    CK(cudaGetLastError());
    enqueued += k;
    batch = std::min(2 * batch, 32);
    CK(cudaMemcpyAsync(host_state, state, sizeof host_state, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
  }
  if (iterations) *iterations = host_state[1];
  if (host_state[0] == 2)
    return h->fail(FEM_GPU_ERR_NOT_CONVERGED, "find_ua_vector_iterative: PCG failed: matrix not positive definite");
  if (n) CK(cudaMemcpyAsync(u_a, x, n * sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (host_state[0] != 1)
    return h->fail(FEM_GPU_ERR_NOT_CONVERGED, "find_ua_vector_iterative: PCG failed: no convergence in %d iterations",
                   max_iter);
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_reactions(fem_gpu_t* h, const double* u_a, const double* u_b, const double* r_b,
                                 double* r_r) {
  if (!h || !u_a || !r_r) return FEM_GPU_ERR_ARGUMENT;
  if (!h->sep_valid) return h->fail(FEM_GPU_ERR_STATE, "call fem_gpu_separate_sparse first");
  cudaStream_t s = h->stream;
  const size_t naa = (size_t)h->sep_n[0], nbb = (size_t)h->sep_n[1];
  DevBuf<double> buf;
  CK(buf.reserve(naa + 3 * nbb + 1, s));
  double* ua = buf.p;
  double* ub = ua + naa;
  double* yba = ub + nbb;
  double* ybb = yba + nbb;
  if (naa) CK(cudaMemcpyAsync(ua, u_a, naa * sizeof(double), cudaMemcpyHostToDevice, s));
  if (nbb) {
    if (u_b) CK(cudaMemcpyAsync(ub, u_b, nbb * sizeof(double), cudaMemcpyHostToDevice, s));
    else CK(cudaMemsetAsync(ub, 0, nbb * sizeof(double), s));
    CK(cudaMemsetAsync(yba, 0, 2 * nbb * sizeof(double), s));
    // y_ba = K_ba u_a, y_bb = K_bb u_b
    k_spmv_add<<<grid_for(nbb * kLanesPerRow, 256), 256, 0, s>>>(nbb, h->sep_rp[2].p, h->sep_ci[2].p, h->sep_v[2].p, ua, yba);
    k_spmv_add<<<grid_for(nbb * kLanesPerRow, 256), 256, 0, s>>>(nbb, h->sep_rp[3].p, h->sep_ci[3].p, h->sep_v[3].p, ub, ybb);
    CK(cudaGetLastError());
  }
  std::vector<double> a(nbb), b(nbb);
  if (nbb) {
    CK(cudaMemcpyAsync(a.data(), yba, nbb * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(b.data(), ybb, nbb * sizeof(double), cudaMemcpyDeviceToHost, s));
  }
  CK(cudaStreamSynchronize(s));
  for (size_t i = 0; i < nbb; ++i) r_r[i] = (a[i] + b[i]) - (r_b ? r_b[i] : 0.0);  // find_r_r_sparse :125-130
  return FEM_GPU_OK;
}
