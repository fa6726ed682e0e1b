// fem_adjoint.cuh -- vector-Jacobian product of the assembly (included by
// fem_gpu.cu, whose handle and element arithmetic it reuses).
//
// For (u_p, lambda_p), p < P, the gradient of F = -sum_p lambda_p^T K u_p with
// respect to every element property theta_e and nodal coordinate is
//     dF/dtheta = -<dK_e/dtheta, W_e>,   W_e = sum_p lambda_{p,e} u_{p,e}^T,
// where lambda_{p,e}, u_{p,e} are the element's DOF slices (global axes).
//   1. u and lambda are transposed to DOF-major (pairs contiguous per DOF);
//   2. W_e is formed per element in shared memory (a small P-deep product);
//   3. one thread per (element, parameter) recomputes the element matrix in
//      forward-mode dual arithmetic seeded on that parameter -- the element
//      matrices are recomputed, never stored -- and contracts dK_e/dtheta with
//      W_e on the fly;
//   4. coordinate contributions are summed per node in a fixed (element) order.
// Parameters: truss E, A, A2; beam E, A, I11, I22, It; plate E, t; nodes x, y, z.

constexpr int kVjpThreads = 128;

// [P][N] -> [N][P] through 32 x 32 shared tiles
__global__ void k_transpose_pairs(const double* __restrict__ in, size_t P, size_t N, double* __restrict__ out) {
  __shared__ double tile[32][33];
  const size_t n0 = (size_t)blockIdx.x * 32, p0 = (size_t)blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const size_t p = p0 + r, n = n0 + threadIdx.x;
    tile[r][threadIdx.x] = (p < P && n < N) ? in[p * N + n] : 0.0;
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const size_t n = n0 + r, p = p0 + threadIdx.x;
    if (n < N && p < P) out[n * P + p] = tile[threadIdx.x][r];
  }
}

// W_e for EPB elements per CTA: ND DOFs per element (NN nodes x NDN DOFs of each node's 6).
template <int ND, int NN, int NDN, int EPB>
__global__ void __launch_bounds__(kVjpThreads) k_vjp_w(size_t n_el, const int32_t* __restrict__ n1,
                                                       const int32_t* __restrict__ n2, const int32_t* __restrict__ n3,
                                                       const int32_t* __restrict__ n4, const double* __restrict__ lamT,
                                                       const double* __restrict__ uT, int P, double* __restrict__ W) {
  extern __shared__ double s_lu[];  // [EPB][2][P][ND]
  const size_t e0 = (size_t)blockIdx.x * EPB;
  const int nloc = (int)min((size_t)EPB, n_el - e0);
  const int32_t* nd[4] = {n1, n2, n3, n4};
  // gather the element DOF slices of lambda and u: (element, array, node, dof, pair), pair fastest
  const int per_el = 2 * NN * NDN * P;
  for (int t = threadIdx.x; t < nloc * per_el; t += blockDim.x) {
    const int el = t / per_el;
    int r = t - el * per_el;
    const int arr = r / (NN * NDN * P);
    r -= arr * NN * NDN * P;
    const int k = r / (NDN * P);
    r -= k * NDN * P;
    const int a = r / P, p = r - a * P;
    const size_t node = (size_t)nd[k][e0 + el];
    const double* src = arr == 0 ? lamT : uT;
    s_lu[(((size_t)el * 2 + arr) * P + p) * ND + k * NDN + a] = src[(6 * node + a) * (size_t)P + p];
  }
  __syncthreads();
  for (int t = threadIdx.x; t < nloc * ND * ND; t += blockDim.x) {
    const int el = t / (ND * ND);
    const int ij = t - el * ND * ND;
    const int i = ij / ND, j = ij - i * ND;
    const double* L = s_lu + (size_t)el * 2 * P * ND;
    const double* U = L + (size_t)P * ND;
    double acc = 0.0;
    for (int p = 0; p < P; ++p) acc = fma(L[p * ND + i], U[p * ND + j], acc);
    W[(e0 + el) * (size_t)(ND * ND) + ij] = acc;
  }
}

// <dK/dtheta, W> of one node-pair block (element orientation), both (i, j) and (j, i)
template <int ND>
__device__ __forceinline__ double contract_pair(const Dual blk[36], int i0, int j0, bool diag,
                                                const double* __restrict__ W) {
  double acc = 0.0;
#pragma unroll
  for (int a = 0; a < 6; ++a)
#pragma unroll
    for (int b = 0; b < 6; ++b) {
      const double d = blk[6 * a + b].d;
      double w = W[(i0 + a) * ND + j0 + b];
      if (!diag) w += W[(j0 + b) * ND + i0 + a];
      acc = fma(d, w, acc);
    }
  return acc;
}

__device__ __forceinline__ void seed3(Dual x[3], const double* v, int base, int dir) {
#pragma unroll
  for (int c = 0; c < 3; ++c) x[c] = Dual(v[c], dir == base + c ? 1.0 : 0.0);
}

template <int I, int J>
__device__ __forceinline__ double plate_pair_dual(const PlateCoreT<Dual>& C, const Dual R[9], bool rot,
                                                  const double* __restrict__ W) {
  Dual blk[36];
  plate_block_ct<I, J>(C, blk);
  if (rot) {
    Dual o[36];
    plate_rotate_block(R, I == J, blk, o);
    return contract_pair<24>(o, 6 * I, 6 * J, I == J, W);
  }
  return contract_pair<24>(blk, 6 * I, 6 * J, I == J, W);
}

// plates: directions 0..11 node coordinates (node k = dir / 3, axis dir % 3), 12 E, 13 t
constexpr int kPlateDirs = 14;
__global__ void __launch_bounds__(64) k_vjp_plate(size_t n_el, NodesView nd, PlateView pl, double abs_tol,
                                                  const double* __restrict__ W, double* __restrict__ g_coord,
                                                  double* __restrict__ g_prop) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= n_el * kPlateDirs) return;
  const size_t e = t / kPlateDirs;
  const int dir = (int)(t - e * kPlateDirs);
  const int nidx[4] = {pl.n1[e], pl.n2[e], pl.n3[e], pl.n4[e]};
  Dual X[4][3];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    double v[3];
    nd.get(nidx[k], v);
    seed3(X[k], v, 3 * k, dir);
  }
  Dual R[9];
  if (!plate_rotation(X[1], X[2], X[3], abs_tol, R)) set_identity(R);
  Dual xl[4] = {0.0, 0.0, 0.0, 0.0}, yl[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    if (i == 2) continue;
    Dual dd[3];
    sub3(X[i], X[2], dd);
    xl[i] = (R[0] * dd[0] + R[1] * dd[1]) + R[2] * dd[2];
    yl[i] = (R[3] * dd[0] + R[4] * dd[1]) + R[5] * dd[2];
  }
  const Dual E(pl.E[e], dir == 12 ? 1.0 : 0.0), th(pl.t[e], dir == 13 ? 1.0 : 0.0);
  PlateCoreT<Dual> C;
  plate_core(xl, yl, E, Dual(pl.nu[e]), th, Dual(pl.ks[e]), C);
  // the rotation can be skipped only when it is the identity and does not move
  bool rot = !is_identity(R);
#pragma unroll
  for (int k = 0; k < 9; ++k) rot = rot || R[k].d != 0.0;
  const double* We = W + e * 576;
  double s = 0.0;
  s += plate_pair_dual<0, 0>(C, R, rot, We);
  s += plate_pair_dual<0, 1>(C, R, rot, We);
  s += plate_pair_dual<0, 2>(C, R, rot, We);
  s += plate_pair_dual<0, 3>(C, R, rot, We);
  s += plate_pair_dual<1, 1>(C, R, rot, We);
  s += plate_pair_dual<1, 2>(C, R, rot, We);
  s += plate_pair_dual<1, 3>(C, R, rot, We);
  s += plate_pair_dual<2, 2>(C, R, rot, We);
  s += plate_pair_dual<2, 3>(C, R, rot, We);
  s += plate_pair_dual<3, 3>(C, R, rot, We);
  if (dir < 12) g_coord[e * 12 + dir] = -s;
  else g_prop[e * 2 + (dir - 12)] = -s;
}

// beams: directions 0..5 node coordinates, 6 E, 7 A, 8 I11, 9 I22, 10 It
constexpr int kBeamDirs = 11;
__global__ void __launch_bounds__(128) k_vjp_beam(size_t n_el, NodesView nd, BeamView b, double rel_tol,
                                                  double abs_tol, const double* __restrict__ W,
                                                  double* __restrict__ g_coord, double* __restrict__ g_prop) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= n_el * kBeamDirs) return;
  const size_t e = t / kBeamDirs;
  const int dir = (int)(t - e * kBeamDirs);
  double v1[3], v2[3];
  nd.get(b.n1[e], v1);
  nd.get(b.n2[e], v2);
  Dual x1[3], x2[3];
  seed3(x1, v1, 0, dir);
  seed3(x2, v2, 3, dir);
  const Dual axis[3] = {Dual(b.ax[e]), Dual(b.ay[e]), Dual(b.az[e])};
  BeamBlocksT<Dual> B;
  if (!beam_blocks(x1, x2, Dual(b.E[e], dir == 6 ? 1.0 : 0.0), Dual(b.nu[e]), Dual(b.A[e], dir == 7 ? 1.0 : 0.0),
                   Dual(b.i11[e], dir == 8 ? 1.0 : 0.0), Dual(b.i22[e], dir == 9 ? 1.0 : 0.0), Dual(b.i12[e]),
                   Dual(b.it[e], dir == 10 ? 1.0 : 0.0), Dual(b.ks[e]), axis, rel_tol, abs_tol, B)) {
    if (dir < 6) g_coord[e * 6 + dir] = 0.0;
    else g_prop[e * 5 + (dir - 6)] = 0.0;
    return;
  }
  const double* We = W + e * 144;
  Dual blk[36];
  double s = 0.0;
  // node block (1,1): [uu ut; ut^T th]
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      blk[6 * a + c] = B.uu[3 * a + c];
      blk[6 * a + 3 + c] = B.ut[3 * a + c];
      blk[6 * (3 + a) + c] = B.ut[3 * c + a];
      blk[6 * (3 + a) + 3 + c] = B.th[3 * a + c];
    }
  s += contract_pair<12>(blk, 0, 0, true, We);
  // node block (1,2): [-uu ut; tu thth2]
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      blk[6 * a + c] = -B.uu[3 * a + c];
      blk[6 * a + 3 + c] = B.ut[3 * a + c];
      blk[6 * (3 + a) + c] = B.tu[3 * a + c];
      blk[6 * (3 + a) + 3 + c] = B.thth2[3 * a + c];
    }
  s += contract_pair<12>(blk, 0, 6, false, We);
  // node block (2,2): [uu -ut; -ut^T th]
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      blk[6 * a + c] = B.uu[3 * a + c];
      blk[6 * a + 3 + c] = -B.ut[3 * a + c];
      blk[6 * (3 + a) + c] = -B.ut[3 * c + a];
      blk[6 * (3 + a) + 3 + c] = B.th[3 * a + c];
    }
  s += contract_pair<12>(blk, 6, 6, true, We);
  if (dir < 6) g_coord[e * 6 + dir] = -s;
  else g_prop[e * 5 + (dir - 6)] = -s;
}

// trusses (3 DOFs per node): directions 0..5 node coordinates, 6 E, 7 A, 8 A2
constexpr int kTrussDirs = 9;
__global__ void __launch_bounds__(128) k_vjp_truss(size_t n_el, NodesView nd, TrussView tv, double abs_tol,
                                                   const double* __restrict__ W, double* __restrict__ g_coord,
                                                   double* __restrict__ g_prop) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= n_el * kTrussDirs) return;
  const size_t e = t / kTrussDirs;
  const int dir = (int)(t - e * kTrussDirs);
  double v1[3], v2[3];
  nd.get(tv.n1[e], v1);
  nd.get(tv.n2[e], v2);
  Dual x1[3], x2[3], g[9];
  seed3(x1, v1, 0, dir);
  seed3(x2, v2, 3, dir);
  double s = 0.0;
  if (truss_block(x1, x2, Dual(tv.E[e], dir == 6 ? 1.0 : 0.0), Dual(tv.A[e], dir == 7 ? 1.0 : 0.0),
                  Dual(tv.A2[e], dir == 8 ? 1.0 : 0.0), abs_tol, g)) {
    const double* We = W + e * 36;
    // blocks (1,1) = g, (1,2) = (2,1) = -g, (2,2) = g over 3 DOFs per node
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const double d = g[3 * a + c].d;
        const double w = We[a * 6 + c] + We[(3 + a) * 6 + 3 + c] - We[a * 6 + 3 + c] - We[(3 + a) * 6 + c];
        s = fma(d, w, s);
      }
  }
  if (dir < 6) g_coord[e * 6 + dir] = -s;
  else g_prop[e * 3 + (dir - 6)] = -s;
}

// node gradients: the coordinate contributions of the node's elements, summed in a fixed order
__global__ void k_vjp_nodes(size_t n_nodes, const int64_t* __restrict__ inc_off, const int64_t* __restrict__ inc,
                            const double* __restrict__ g_coord, double* __restrict__ g_xyz) {
  const size_t n = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (n >= n_nodes) return;
  double gx = 0.0, gy = 0.0, gz = 0.0;
  for (int64_t k = inc_off[n]; k < inc_off[n + 1]; ++k) {
    const int64_t base = inc[k];
    gx += g_coord[base];
    gy += g_coord[base + 1];
    gz += g_coord[base + 2];
  }
  g_xyz[3 * n] = gx;
  g_xyz[3 * n + 1] = gy;
  g_xyz[3 * n + 2] = gz;
}

namespace {

// node -> coordinate-contribution bases (trusses, then beams, then plates; element order)
int vjp_incidence(fem_gpu* h) {
  if (h->vjp_inc_valid) return FEM_GPU_OK;
  const size_t n = h->n_nodes;
  std::vector<int32_t> t1(h->nt), t2(h->nt), b1(h->nbm), b2(h->nbm), p[4];
  CK(cudaMemcpyAsync(t1.data(), h->t_n1.p, h->nt * 4, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(t2.data(), h->t_n2.p, h->nt * 4, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(b1.data(), h->b_n1.p, h->nbm * 4, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(b2.data(), h->b_n2.p, h->nbm * 4, cudaMemcpyDeviceToHost, h->stream));
  const int32_t* dp[4] = {h->p_n1.p, h->p_n2.p, h->p_n3.p, h->p_n4.p};
  for (int k = 0; k < 4; ++k) {
    p[k].resize(h->np);
    CK(cudaMemcpyAsync(p[k].data(), dp[k], h->np * 4, cudaMemcpyDeviceToHost, h->stream));
  }
  CK(cudaStreamSynchronize(h->stream));
  const int64_t off_b = (int64_t)h->nt * 6, off_p = off_b + (int64_t)h->nbm * 6;
  std::vector<int64_t> cnt(n + 1, 0);
  for (size_t e = 0; e < h->nt; ++e) cnt[t1[e] + 1]++, cnt[t2[e] + 1]++;
  for (size_t e = 0; e < h->nbm; ++e) cnt[b1[e] + 1]++, cnt[b2[e] + 1]++;
  for (int k = 0; k < 4; ++k)
    for (size_t e = 0; e < h->np; ++e) cnt[p[k][e] + 1]++;
  for (size_t i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
  std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1), inc((size_t)cnt[n]);
  for (size_t e = 0; e < h->nt; ++e) {
    inc[fill[t1[e]]++] = (int64_t)e * 6;
    inc[fill[t2[e]]++] = (int64_t)e * 6 + 3;
  }
  for (size_t e = 0; e < h->nbm; ++e) {
    inc[fill[b1[e]]++] = off_b + (int64_t)e * 6;
    inc[fill[b2[e]]++] = off_b + (int64_t)e * 6 + 3;
  }
  for (size_t e = 0; e < h->np; ++e)
    for (int k = 0; k < 4; ++k) inc[fill[p[k][e]]++] = off_p + (int64_t)e * 12 + 3 * k;
  CK(h->vjp_inc_off.reserve(n + 1, h->stream));
  CK(h->vjp_inc.reserve(inc.size() + 1, h->stream));
  CK(cudaMemcpyAsync(h->vjp_inc_off.p, cnt.data(), (n + 1) * 8, cudaMemcpyHostToDevice, h->stream));
  if (!inc.empty()) CK(cudaMemcpyAsync(h->vjp_inc.p, inc.data(), inc.size() * 8, cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  h->vjp_inc_valid = true;
  return FEM_GPU_OK;
}

int vjp_launch(fem_gpu* h, const double* d_u, const double* d_lam, int P) {
  cudaStream_t s = h->stream;
  const size_t N = (size_t)h->nodes_number * 6;
  CK(h->vjp_uT.reserve(N * P + 1, s));
  CK(h->vjp_lT.reserve(N * P + 1, s));
  const dim3 tb(32, 8), tg((unsigned)((N + 31) / 32), (unsigned)((P + 31) / 32));
  k_transpose_pairs<<<tg, tb, 0, s>>>(d_u, (size_t)P, N, h->vjp_uT.p);
  k_transpose_pairs<<<tg, tb, 0, s>>>(d_lam, (size_t)P, N, h->vjp_lT.p);
  const size_t wt = h->nt * 36, wb = h->nbm * 144, wp = h->np * 576;
  CK(h->vjp_W.reserve(wt + wb + wp + 1, s));
  const size_t ct = h->nt * 6, cb = h->nbm * 6, cp = h->np * 12;
  CK(h->vjp_gc.reserve(ct + cb + cp + 1, s));
  CK(h->vjp_gp.reserve(h->nt * 3 + h->nbm * 5 + h->np * 2 + 1, s));
  double* Wt = h->vjp_W.p;
  double* Wb = Wt + wt;
  double* Wp = Wb + wb;
  double* gct = h->vjp_gc.p;
  double* gcb = gct + ct;
  double* gcp = gcb + cb;
  double* gpt = h->vjp_gp.p;
  double* gpb = gpt + h->nt * 3;
  double* gpp = gpb + h->nbm * 5;
  const NodesView nd = h->nodes();
  if (h->nt) {
    const size_t smem = (size_t)4 * 2 * P * 6 * sizeof(double);
    CK(cudaFuncSetAttribute(k_vjp_w<6, 2, 3, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_vjp_w<6, 2, 3, 4><<<grid_for(h->nt, 4), kVjpThreads, smem, s>>>(h->nt, h->t_n1.p, h->t_n2.p, nullptr, nullptr,
                                                                     h->vjp_lT.p, h->vjp_uT.p, P, Wt);
    k_vjp_truss<<<grid_for(h->nt * kTrussDirs, 128), 128, 0, s>>>(h->nt, nd, h->trusses(), h->abs_tol, Wt, gct, gpt);
  }
  if (h->nbm) {
    const size_t smem = (size_t)2 * 2 * P * 12 * sizeof(double);
    CK(cudaFuncSetAttribute(k_vjp_w<12, 2, 6, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_vjp_w<12, 2, 6, 2><<<grid_for(h->nbm, 2), kVjpThreads, smem, s>>>(h->nbm, h->b_n1.p, h->b_n2.p, nullptr,
                                                                       nullptr, h->vjp_lT.p, h->vjp_uT.p, P, Wb);
    k_vjp_beam<<<grid_for(h->nbm * kBeamDirs, 128), 128, 0, s>>>(h->nbm, nd, h->beams(), h->rel_tol, h->abs_tol, Wb,
                                                                  gcb, gpb);
  }
  if (h->np) {
    const size_t smem = (size_t)1 * 2 * P * 24 * sizeof(double);
    CK(cudaFuncSetAttribute(k_vjp_w<24, 4, 6, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_vjp_w<24, 4, 6, 1><<<grid_for(h->np, 1), kVjpThreads, smem, s>>>(h->np, h->p_n1.p, h->p_n2.p, h->p_n3.p,
                                                                      h->p_n4.p, h->vjp_lT.p, h->vjp_uT.p, P, Wp);
    k_vjp_plate<<<grid_for(h->np * kPlateDirs, 64), 64, 0, s>>>(h->np, nd, h->plates(), h->abs_tol, Wp, gcp, gpp);
  }
  CK(h->vjp_gxyz.reserve(h->n_nodes * 3 + 1, s));
  if (h->n_nodes)
    k_vjp_nodes<<<grid_for(h->n_nodes, 256), 256, 0, s>>>(h->n_nodes, h->vjp_inc_off.p, h->vjp_inc.p, h->vjp_gc.p,
                                                          h->vjp_gxyz.p);
  CK(cudaGetLastError());
  return FEM_GPU_OK;
}

}  // namespace

extern "C" int fem_gpu_vjp(fem_gpu_t* h, const double* u, const double* lam, int npairs, double* g_truss,
                           double* g_beam, double* g_plate, double* g_xyz) {
  if (!h || !u || !lam || npairs < 1 || npairs > 512) return FEM_GPU_ERR_ARGUMENT;
  int st = ensure_ready(h);
  if (st) return st;
  st = vjp_incidence(h);
  if (st) return st;
  const size_t N = (size_t)h->nodes_number * 6, P = (size_t)npairs;
  CK(h->vjp_in.reserve(2 * N * P + 1, h->stream));
  CK(cudaMemcpyAsync(h->vjp_in.p, u, N * P * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->vjp_in.p + N * P, lam, N * P * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CK(cudaEventRecord(h->ev[0], h->stream));
  st = vjp_launch(h, h->vjp_in.p, h->vjp_in.p + N * P, npairs);
  if (st) return st;
  CK(cudaEventRecord(h->ev[1], h->stream));
  double* gp = h->vjp_gp.p;
  if (g_truss && h->nt) CK(cudaMemcpyAsync(g_truss, gp, h->nt * 3 * 8, cudaMemcpyDeviceToHost, h->stream));
  if (g_beam && h->nbm)
    CK(cudaMemcpyAsync(g_beam, gp + h->nt * 3, h->nbm * 5 * 8, cudaMemcpyDeviceToHost, h->stream));
  if (g_plate && h->np)
    CK(cudaMemcpyAsync(g_plate, gp + h->nt * 3 + h->nbm * 5, h->np * 2 * 8, cudaMemcpyDeviceToHost, h->stream));
  if (g_xyz && h->n_nodes)
    CK(cudaMemcpyAsync(g_xyz, h->vjp_gxyz.p, h->n_nodes * 3 * 8, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaEventElapsedTime(&h->t_vjp_ms, h->ev[0], h->ev[1]));
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_vjp_last_ms(fem_gpu_t* h, float* ms) {
  if (!h || !ms) return FEM_GPU_ERR_ARGUMENT;
  *ms = h->t_vjp_ms;
  return FEM_GPU_OK;
}
