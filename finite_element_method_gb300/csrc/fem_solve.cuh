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
// abs_tol), checked after every iteration.  Products are a few lanes per CSR row
// and dot products a fixed two-level tree, so results repeat run to run.

constexpr int kDotBlocks = 1024, kDotThreads = 256;

// y[i] = sum_j K[i][j] x[j], or a (s[i] - that sum) when s is given.  kLanesPerRow lanes per row (strided
// partial sums, then a two-step shuffle tree): FP64 adds are scarce on this GPU, so a whole warp per ~20-entry
// row, with its five-step tree, would leave the FP64 pipe, not HBM, as the limit.
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

// per-block partial sums of x[i] * y[i] (fixed order), then one block sums the partials
__global__ void __launch_bounds__(kDotThreads) k_dot_partial(size_t n, const double* __restrict__ x,
                                                             const double* __restrict__ y, double* __restrict__ part) {
  __shared__ double sh[kDotThreads];
  double acc = 0.0;
  for (size_t i = blockIdx.x * (size_t)kDotThreads + threadIdx.x; i < n; i += (size_t)gridDim.x * kDotThreads)
    acc = fma(x[i], y[i], acc);
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kDotThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}
__global__ void __launch_bounds__(kDotThreads) k_dot_final(int n_part, const double* __restrict__ part,
                                                           double* __restrict__ out) {
  __shared__ double sh[kDotThreads];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n_part; i += kDotThreads) acc += part[i];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kDotThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

// preconditioner blocks: the free DOFs of one node (consecutive in the a list); start of each block per DOF
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
// blocks of size 1 are the Jacobi preconditioner.  inv: 36 doubles per block
__global__ void k_block_inverse(size_t nblk, const uint32_t* __restrict__ start, size_t n,
                                const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                const double* __restrict__ v, double* __restrict__ inv, int* singular) {
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
  for (int i = 0; i < 36; ++i) inv[36 * b + i] = X[i];
}

// z = M^-1 r, one thread per block
__global__ void k_block_apply(size_t nblk, const uint32_t* __restrict__ start, size_t n,
                              const double* __restrict__ inv, const double* __restrict__ r, double* __restrict__ z) {
  const size_t b = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (b >= nblk) return;
  const uint32_t s = start[b], e = b + 1 < nblk ? start[b + 1] : (uint32_t)n;
  const int m = (int)(e - s);
  double rr[6];
  for (int j = 0; j < m; ++j) rr[j] = r[s + j];
  for (int i = 0; i < m; ++i) {
    double acc = 0.0;
    for (int j = 0; j < m; ++j) acc = fma(inv[36 * b + 6 * i + j], rr[j], acc);
    z[s + i] = acc;
  }
}

// the recurrence's scalars stay on the device: sc[kRz] = r.z, sc[kPq] = p.Aq, sc[kRr] = r.r, sc[kRzNew]
enum { kRz = 0, kPq = 1, kRr = 2, kRzNew = 3, kAlpha = 4, kBeta = 5, kScalars = 6 };

// alpha = rz / pq (a non-positive pq is recorded: the matrix is not positive definite)
__global__ void k_cg_alpha(double* sc, int* bad) {
  if (!(sc[kPq] > 0.0)) *bad = 1;
  sc[kAlpha] = sc[kRz] / sc[kPq];
}
// beta = rz_new / rz, then rz = rz_new
__global__ void k_cg_beta(double* sc) {
  sc[kBeta] = sc[kRzNew] / sc[kRz];
  sc[kRz] = sc[kRzNew];
}

// x += alpha p, r -= alpha q
__global__ void k_cg_update(size_t n, const double* __restrict__ sc, const double* __restrict__ p,
                            const double* __restrict__ q, double* __restrict__ x, double* __restrict__ r) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double alpha = sc[kAlpha];
  x[i] = fma(alpha, p[i], x[i]);
  r[i] = fma(-alpha, q[i], r[i]);
}

// p = z + beta p
__global__ void k_cg_direction(size_t n, const double* __restrict__ sc, const double* __restrict__ z,
                               double* __restrict__ p) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  p[i] = fma(sc[kBeta], p[i], z[i]);
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

namespace {

// sc[slot] = x . y on the stream (no host synchronisation)
void dot_enqueue(fem_gpu* h, size_t n, const double* x, const double* y, int slot) {
  cudaStream_t s = h->stream;
  const int nb = (int)std::min<size_t>(kDotBlocks, std::max<size_t>(1, (n + kDotThreads - 1) / kDotThreads));
  k_dot_partial<<<nb, kDotThreads, 0, s>>>(n, x, y, h->pcg_part.p);
  k_dot_final<<<1, kDotThreads, 0, s>>>(nb, h->pcg_part.p, h->pcg_scal.p + slot);
}

int read_scalar(fem_gpu* h, int slot, double* out) {
  CK(cudaMemcpyAsync(out, h->pcg_scal.p + slot, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return FEM_GPU_OK;
}

}  // namespace

extern "C" int fem_gpu_solve_pcg(fem_gpu_t* h, const double* r_a, const double* u_b, int block_jacobi, int max_iter,
                                 double* u_a, int* iterations) {
  if (!h || !r_a || !u_a || max_iter < 0) return FEM_GPU_ERR_ARGUMENT;
  if (!h->sep_valid) return h->fail(FEM_GPU_ERR_STATE, "call fem_gpu_separate_sparse first");
  cudaStream_t s = h->stream;
  const size_t n = (size_t)h->sep_n[0], nbb = (size_t)h->sep_n[1];
  if (iterations) *iterations = 0;
  CK(h->pcg_vec.reserve(6 * n + nbb + 1, s));
  CK(h->pcg_part.reserve(kDotBlocks, s));
  CK(h->pcg_scal.reserve(kScalars, s));
  double* x = h->pcg_vec.p;
  double* r = x + n;
  double* z = r + n;
  double* p = z + n;
  double* q = p + n;
  double* ra = q + n;
  double* ub = ra + n;
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
    int st = cub_call(h, [&](void* tmp, size_t& bytes) {
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
  CK(h->pcg_inv.reserve(36 * nblk + 1, s));
  CK(h->flag.reserve(1, s));
  CK(cudaMemsetAsync(h->flag.p, 0, sizeof(int), s));
  if (nblk)
    k_block_inverse<<<grid_for(nblk, 128), 128, 0, s>>>(nblk, h->pcg_blk.p, n, h->sep_rp[0].p, h->sep_ci[0].p,
                                                        h->sep_v[0].p, h->pcg_inv.p, h->flag.p);
  int singular = 0;
  CK(cudaMemcpyAsync(&singular, h->flag.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (singular) return h->fail(FEM_GPU_ERR_NOT_CONVERGED, "find_ua_vector_iterative: PCG failed: singular preconditioner");
  // PCG: one host synchronisation per iteration, on the residual norm
  double bb = 0.0;
  dot_enqueue(h, n, r, r, kRr);
  int st = read_scalar(h, kRr, &bb);
  if (st) return st;
  const double tol = std::max(h->rel_tol * sqrt(bb), h->abs_tol);
  int it = 0;
  bool done = !(sqrt(bb) > tol);
  if (!done) {
    k_block_apply<<<grid_for(nblk, 128), 128, 0, s>>>(nblk, h->pcg_blk.p, n, h->pcg_inv.p, r, z);
    CK(cudaMemcpyAsync(p, z, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    dot_enqueue(h, n, r, z, kRz);
  }
  CK(cudaMemsetAsync(h->flag.p, 0, sizeof(int), s));
  while (!done && it < max_iter) {
    k_spmv<<<grid_for(n * kLanesPerRow, 256), 256, 0, s>>>(n, h->sep_rp[0].p, h->sep_ci[0].p, h->sep_v[0].p, p,
                                                            nullptr, 1.0, q);
    dot_enqueue(h, n, p, q, kPq);
    k_cg_alpha<<<1, 1, 0, s>>>(h->pcg_scal.p, h->flag.p);
    k_cg_update<<<grid_for(n, 256), 256, 0, s>>>(n, h->pcg_scal.p, p, q, x, r);
    ++it;
    dot_enqueue(h, n, r, r, kRr);
    double rr = 0.0;
    int bad = 0;
    CK(cudaMemcpyAsync(&bad, h->flag.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    st = read_scalar(h, kRr, &rr);
    if (st) return st;
    if (bad)
      return h->fail(FEM_GPU_ERR_NOT_CONVERGED, "find_ua_vector_iterative: PCG failed: matrix not positive definite");
    if (!(sqrt(rr) > tol)) {
      done = true;
      break;
    }
    k_block_apply<<<grid_for(nblk, 128), 128, 0, s>>>(nblk, h->pcg_blk.p, n, h->pcg_inv.p, r, z);
    dot_enqueue(h, n, r, z, kRzNew);
    k_cg_beta<<<1, 1, 0, s>>>(h->pcg_scal.p);
    k_cg_direction<<<grid_for(n, 256), 256, 0, s>>>(n, h->pcg_scal.p, z, p);
  }
  CK(cudaGetLastError());
  if (n) CK(cudaMemcpyAsync(u_a, x, n * sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (iterations) *iterations = it;
  if (!done)
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
