// fem_adjoint.cuh -- vector-Jacobian product of the assembly (included by
// fem_gpu.cu, whose handle and element arithmetic it reuses).
//
// For (u_p, lambda_p), p < P, the gradient of F = -sum_p lambda_p^T K u_p with
// respect to every element property theta_e and nodal coordinate is
//     dF/dtheta = -<dK_e/dtheta, W_e>,   W_e = sum_p lambda_{p,e} u_{p,e}^T,
// where lambda_{p,e}, u_{p,e} are the element's DOF slices (global axes).  K_e
// is symmetric, so only Ws = W + W^T matters, and Ws restricted to an element
// is a set of global node-pair blocks: Ws(I, J) = sum_p (lambda_I u_J^T +
// u_I lambda_J^T), shared by every element that couples nodes I and J.
//   1. u and lambda are transposed to DOF-major (pairs contiguous per DOF);
//   2. Ws is formed once per block of the stiffness pattern (a sampled
//      dense-dense product: 36 entries x 2P fused multiply-adds per block);
//   3. the element kernels recompute their element matrices in forward-mode
//      dual arithmetic -- recomputed, never stored -- and contract the
//      derivatives with their blocks of Ws;
//   4. coordinate contributions are summed per node in a fixed (element) order.
// Parameters: truss E, A, A2; beam E, A, I11, I22, It; plate E, t; nodes x, y, z.

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

// the stiffness block of every element node pair: the block whose sorted range holds the pair's slot
__global__ void k_pair_blocks(size_t n, const uint32_t* __restrict__ slot, const uint32_t* __restrict__ blk_start,
                              size_t n_blocks, uint32_t* __restrict__ pblk) {
  const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t s = slot[k];
  size_t lo = 0, hi = n_blocks;  // last block with blk_start <= s
  while (hi - lo > 1) {
    const size_t mid = (lo + hi) >> 1;
    if (blk_start[mid] <= s) lo = mid;
    else hi = mid;
  }
  pblk[k] = (uint32_t)lo;
}

// Ws(I, J) for every pattern block, one thread per entry (a, c), rows the DOFs of I = blk_I <= J = blk_J:
//   Ws[b][6a + c] = sum_p lambda[6I + a][p] u[6J + c][p] + u[6I + a][p] lambda[6J + c][p]
constexpr int kWsBlocksPerCta = 8;
__global__ void __launch_bounds__(36 * kWsBlocksPerCta) k_vjp_ws(size_t n_blocks, const int32_t* __restrict__ blk_I,
                                                                 const int32_t* __restrict__ blk_J,
                                                                 const double* __restrict__ lamT,
                                                                 const double* __restrict__ uT, int P,
                                                                 double* __restrict__ Ws) {
  const size_t b = (size_t)blockIdx.x * kWsBlocksPerCta + threadIdx.x / 36;
  if (b >= n_blocks) return;
  const int ac = threadIdx.x % 36, a = ac / 6, c = ac % 6;
  const size_t I = (size_t)blk_I[b], J = (size_t)blk_J[b];
  const double* li = lamT + (6 * I + a) * (size_t)P;
  const double* ui = uT + (6 * I + a) * (size_t)P;
  const double* lj = lamT + (6 * J + c) * (size_t)P;
  const double* uj = uT + (6 * J + c) * (size_t)P;
  double acc0 = 0.0, acc1 = 0.0;
  int p = 0;
  if ((P & 1) == 0) {  // rows start 16-byte aligned when P is even
    for (; p < P; p += 2) {
      const double2 l2 = __ldg(reinterpret_cast<const double2*>(li + p));
      const double2 u2 = __ldg(reinterpret_cast<const double2*>(ui + p));
      const double2 m2 = __ldg(reinterpret_cast<const double2*>(lj + p));
      const double2 v2 = __ldg(reinterpret_cast<const double2*>(uj + p));
      acc0 = fma(l2.x, v2.x, acc0);
      acc1 = fma(u2.x, m2.x, acc1);
      acc0 = fma(l2.y, v2.y, acc0);
      acc1 = fma(u2.y, m2.y, acc1);
    }
  } else {
    for (; p < P; ++p) {
      acc0 = fma(li[p], uj[p], acc0);
      acc1 = fma(ui[p], lj[p], acc1);
    }
  }
  Ws[b * 36 + ac] = acc0 + acc1;
}

// entry (a, c) of Ws between DOF a of global node gi and DOF c of global node gj, from the stored block
// (rows = the lower node index); Ws is symmetric, so the other orientation is the transpose
__device__ __forceinline__ double ws_at(const double* __restrict__ blk, int32_t gi, int32_t gj, int a, int c) {
  return gi <= gj ? blk[6 * a + c] : blk[6 * c + a];
}

// <dK/dtheta, W> of one node-pair block (element orientation, element nodes gi, gj): sum d Ws over the
// block, halved on the diagonal (there d is symmetric and Ws counts both orientations)
__device__ __forceinline__ double contract_ws(const Dual blk[36], const double* __restrict__ ws, int32_t gi,
                                              int32_t gj, bool diag) {
  double acc = 0.0;
#pragma unroll
  for (int a = 0; a < 6; ++a)
#pragma unroll
    for (int c = 0; c < 6; ++c) acc = fma(blk[6 * a + c].d, ws_at(ws, gi, gj, a, c), acc);
  return diag ? 0.5 * acc : acc;
}

__device__ __forceinline__ void seed3(Dual x[3], const double* v, int base, int dir) {
#pragma unroll
  for (int c = 0; c < 3; ++c) x[c] = Dual(v[c], dir == base + c ? 1.0 : 0.0);
}

// Plates, in the element's local frame.  With T = blockdiag(R) (eight 3x3
// copies), S = T W_e T^T and Sh = S + S^T = T (W_e + W_e^T) T^T, the
// contraction is f = <K_g, W_e> = <K_l, S> = 1/2 <K_l, Sh>, and its gradient
// has two parts:
//  * through K_l -- the local coordinates xl, yl of nodes 1, 2, 4 (node 3 is
//    the local origin), E and t: eight forward-mode directions, one per lane
//    of the plate's 8-lane group, each contracted with Sh on K_l's structural
//    entries (13 or 14 of a node-pair block's 36; K_l is zero elsewhere, so
//    no rotated dual blocks are formed);
//  * through R -- with omega = dR R^T (dT = blockdiag(omega) T):
//    df = <omega, M>, M = sum_k (K_l Sh)_kk over the eight 3x3 diagonal
//    blocks, plus the local coordinates' own dependence on R, <H, dR> with
//    rows 0, 1 of H = sum_i (df/dxl_i, df/dyl_i) (x_i - x_3)^T.
//    R depends on nodes 2, 3, 4 through (x4 - x3) x (x2 - x3) only, so
//    dR/dx3 = -(dR/dx2 + dR/dx4): six dual rotations.
// The chain rule back to global coordinates then uses xl_i = R_0 . (x_i - x_3),
// yl_i = R_1 . (x_i - x_3).  Lanes: 0..5 seed xl1, yl1, xl2, yl2, xl4, yl4;
// 6 seeds t; 7 seeds E.
constexpr int kPlateLanes = 8;
constexpr int kPlatesPerCta = 4;  // one warp
constexpr int kPlateKl = 134;     // structural entries of the ten upper node-pair blocks

// upper node-pair block b (0..9) = (I, J): (0,0) (0,1) (0,2) (0,3) (1,1) (1,2) (1,3) (2,2) (2,3) (3,3)
__host__ __device__ constexpr int plate_pair_i(int b) { return b < 4 ? 0 : b < 7 ? 1 : b < 9 ? 2 : 3; }
__host__ __device__ constexpr int plate_pair_j(int b) { return b < 4 ? b : b < 7 ? b - 3 : b < 9 ? b - 5 : 3; }
// first structural entry of block b in the packed list (diagonal blocks 14 entries, others 13)
__host__ __device__ constexpr int plate_pair_off(int b) {
  return 13 * b + (b > 0 ? 1 : 0) + (b > 4 ? 1 : 0) + (b > 7 ? 1 : 0);
}
// k-th structural entry (row-major index in the 6x6 block): u-v membrane, w-thx-thy plate, thz-thz drilling
__host__ __device__ constexpr int plate_en(int k) {
  return k < 2 ? k : k < 4 ? k + 4 : k < 7 ? k + 10 : k < 10 ? k + 13 : k < 13 ? k + 16 : 35;
}

// <dK_l/dtheta, Sh> over block B's structural entries (halved on diagonal blocks); the block's
// values go to Kl on the lane that owns the block
template <int B>
__device__ __forceinline__ double plate_local_pair(const PlateCoreT<Dual>& C, const double* __restrict__ Sh,
                                                   double* __restrict__ Kl, bool owner) {
  constexpr int I = plate_pair_i(B), J = plate_pair_j(B), NE = I == J ? 14 : 13;
  Dual blk[36];
  plate_block_ct<I, J>(C, blk);
  double acc = 0.0;
#pragma unroll
  for (int k = 0; k < NE; ++k) {
    const int en = plate_en(k);
    acc = fma(blk[en].d, Sh[(6 * I + en / 6) * 24 + 6 * J + en % 6], acc);
    if (owner) Kl[plate_pair_off(B) + k] = blk[en].v;
  }
  return I == J ? 0.5 * acc : acc;
}

__global__ void __launch_bounds__(kPlateLanes* kPlatesPerCta) k_vjp_plate(size_t n_el, NodesView nd, PlateView pl,
                                                                          double abs_tol, const double* __restrict__ Ws,
                                                                          const uint32_t* __restrict__ pblk,
                                                                          double* __restrict__ g_coord,
                                                                          double* __restrict__ g_prop) {
  __shared__ double s_sh[kPlatesPerCta][576];
  __shared__ double s_kl[kPlatesPerCta][kPlateKl];
  __shared__ double s_m[kPlatesPerCta][kPlateLanes][9];
  __shared__ double s_phi[kPlatesPerCta][kPlateLanes];
  __shared__ double s_rot[kPlatesPerCta][kPlateLanes];
  const int grp = threadIdx.x / kPlateLanes, lane = threadIdx.x % kPlateLanes;
  const size_t e = (size_t)blockIdx.x * kPlatesPerCta + grp;
  const bool live = e < n_el;
  const size_t ec = live ? e : n_el - 1;  // tail groups recompute the last plate and store nothing
  double* Sh = s_sh[grp];
  double* Kl = s_kl[grp];

  // geometry (values): R with the forward kernel's identity fast path, local coordinates
  const int nidx[4] = {pl.n1[ec], pl.n2[ec], pl.n3[ec], pl.n4[ec]};
  double X[4][3];
#pragma unroll
  for (int k = 0; k < 4; ++k) nd.get(nidx[k], X[k]);
  double R[9];
  if (!plate_rotation(X[1], X[2], X[3], abs_tol, R)) set_identity(R);
  const bool ident = is_identity(R);
  double xlv[4], ylv[4], dv[4][3];
#pragma unroll
  for (int i = 0; i < 4; ++i) sub3(X[i], X[2], dv[i]);
  plate_local_xy(X, R, ident, xlv, ylv);

  // 1. Sh = R Ws R^T by 3x3 sub-blocks, Ws from the element's stiffness blocks; lane p fills sub-block row p
  {
    const int p = lane;
#pragma unroll 1
    for (int q = 0; q < 8; ++q) {
      const int ie = p / 2, je = q / 2;
      const double* wb = Ws + (size_t)pblk[ec * 10 + (ie <= je ? ut4(ie, je) : ut4(je, ie))] * 36;
      double ws[9];
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) ws[3 * a + b] = ws_at(wb, nidx[ie], nidx[je], 3 * (p % 2) + a, 3 * (q % 2) + b);
      if (!ident) {
        double t[9];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int c = 0; c < 3; ++c) t[3 * a + c] = (ws[3 * a] * R[3 * c] + ws[3 * a + 1] * R[3 * c + 1]) + ws[3 * a + 2] * R[3 * c + 2];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int c = 0; c < 3; ++c) ws[3 * a + c] = (R[3 * a] * t[c] + R[3 * a + 1] * t[3 + c]) + R[3 * a + 2] * t[6 + c];
      }
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) Sh[(3 * p + a) * 24 + 3 * q + b] = ws[3 * a + b];
    }
  }
  __syncthreads();

  // 2. one forward-mode direction per lane through K_l, contracted with Sh
  {
    Dual xl[4], yl[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int s = i == 3 ? 2 : i;  // seed slot of node i (node 3 is the origin: none)
      xl[i] = Dual(xlv[i], (i != 2 && lane == 2 * s) ? 1.0 : 0.0);
      yl[i] = Dual(ylv[i], (i != 2 && lane == 2 * s + 1) ? 1.0 : 0.0);
    }
    const Dual E(pl.E[ec], lane == 7 ? 1.0 : 0.0), th(pl.t[ec], lane == 6 ? 1.0 : 0.0);
    PlateCoreT<Dual> C;
    plate_core(xl, yl, E, Dual(pl.nu[ec]), th, Dual(pl.ks[ec]), C);
    double phi = 0.0;
    phi += plate_local_pair<0>(C, Sh, Kl, lane == 0);
    phi += plate_local_pair<1>(C, Sh, Kl, lane == 1);
    phi += plate_local_pair<2>(C, Sh, Kl, lane == 2);
    phi += plate_local_pair<3>(C, Sh, Kl, lane == 3);
    phi += plate_local_pair<4>(C, Sh, Kl, lane == 4);
    phi += plate_local_pair<5>(C, Sh, Kl, lane == 5);
    phi += plate_local_pair<6>(C, Sh, Kl, lane == 6);
    phi += plate_local_pair<7>(C, Sh, Kl, lane == 7);
    phi += plate_local_pair<8>(C, Sh, Kl, lane == 0);
    phi += plate_local_pair<9>(C, Sh, Kl, lane == 1);
    s_phi[grp][lane] = phi;
  }
  __syncthreads();

  // 3. M = sum_k (K_l Sh)_kk: lane l takes the structural entries of blocks l and l + 8
  {
    double* M = s_m[grp][lane];
#pragma unroll
    for (int k = 0; k < 9; ++k) M[k] = 0.0;
#pragma unroll 1
    for (int B = lane; B < 10; B += kPlateLanes) {
      const int I = plate_pair_i(B), J = plate_pair_j(B), ne = I == J ? 14 : 13, off = plate_pair_off(B);
#pragma unroll 1
      for (int k = 0; k < ne; ++k) {
        const int en = plate_en(k), r = en / 6, c = en % 6;
        const double kv = Kl[off + k];
        const int p = 2 * I + r / 3, q = 2 * J + c / 3, a = r % 3, cc = c % 3;
        // K{p,q}[a][cc] = kv adds kv Sh{q,p}[cc][:] to row a
#pragma unroll
        for (int b = 0; b < 3; ++b) M[3 * a + b] = fma(kv, Sh[(3 * q + cc) * 24 + 3 * p + b], M[3 * a + b]);
        // off-diagonal blocks: K{q,p}[cc][a] = kv adds kv Sh{p,q}[a][:] to row cc
        if (I != J)
#pragma unroll
          for (int b = 0; b < 3; ++b) M[3 * cc + b] = fma(kv, Sh[(3 * p + a) * 24 + 3 * q + b], M[3 * cc + b]);
      }
    }
  }
  __syncthreads();

  // 4. rotation directions: lanes 0..5 = x, y, z of node 2, then of node 4 (lanes 6, 7 repeat lane 0)
  {
    const int dir = lane < 6 ? lane : 0;
    const int node = dir < 3 ? 1 : 3, axis = dir % 3;
    double Mt[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      double s = 0.0;
#pragma unroll
      for (int l = 0; l < kPlateLanes; ++l) s += s_m[grp][l][k];
      Mt[k] = s;
    }
    const double* phi = s_phi[grp];
    const int slot_of[3] = {0, 1, 3};
    double H[6];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      double hx = 0.0, hy = 0.0;
#pragma unroll
      for (int s = 0; s < 3; ++s) {
        hx = fma(phi[2 * s], dv[slot_of[s]][j], hx);
        hy = fma(phi[2 * s + 1], dv[slot_of[s]][j], hy);
      }
      H[j] = hx;
      H[3 + j] = hy;
    }
    Dual Xd[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int c = 0; c < 3; ++c) Xd[k][c] = Dual(X[k + 1][c], (k + 1 == node && c == axis) ? 1.0 : 0.0);
    Dual Rd[9];
    if (!plate_rotation(Xd[0], Xd[1], Xd[2], abs_tol, Rd)) set_identity(Rd);
    double r = 0.0;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        // omega = dR R^T
        const double om = (Rd[3 * a].d * R[3 * b] + Rd[3 * a + 1].d * R[3 * b + 1]) + Rd[3 * a + 2].d * R[3 * b + 2];
        r = fma(om, Mt[3 * a + b], r);
      }
#pragma unroll
    for (int j = 0; j < 3; ++j) r = fma(H[j], Rd[j].d, fma(H[3 + j], Rd[3 + j].d, r));
    s_rot[grp][lane] = r;
  }
  __syncthreads();

  // 5. outputs: lane l writes entries l and l + 8 of (12 coordinates, E, t)
  if (live) {
    const double* phi = s_phi[grp];
    const double* rot = s_rot[grp];
#pragma unroll
    for (int o = lane; o < 14; o += kPlateLanes) {
      double v;
      if (o >= 12) {
        v = phi[o == 12 ? 7 : 6];
        g_prop[e * 2 + (o - 12)] = -v;
        continue;
      }
      const int node = o / 3, j = o % 3;
      if (node == 2) {
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < 3; ++q) s += phi[2 * q] * R[j] + phi[2 * q + 1] * R[3 + j];
        v = -s - (rot[j] + rot[3 + j]);
      } else {
        const int slot = node == 3 ? 2 : node;
        v = phi[2 * slot] * R[j] + phi[2 * slot + 1] * R[3 + j];
        if (node == 1) v += rot[j];
        if (node == 3) v += rot[3 + j];
      }
      g_coord[e * 12 + o] = -v;
    }
  }
}

// beams: directions 0..5 node coordinates, 6 E, 7 A, 8 I11, 9 I22, 10 It
constexpr int kBeamDirs = 11;
__global__ void __launch_bounds__(128) k_vjp_beam(size_t n_el, NodesView nd, BeamView b, double rel_tol,
                                                  double abs_tol, const double* __restrict__ Ws,
                                                  const uint32_t* __restrict__ pblk, double* __restrict__ g_coord,
                                                  double* __restrict__ g_prop) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= n_el * kBeamDirs) return;
  const size_t e = t / kBeamDirs;
  const int dir = (int)(t - e * kBeamDirs);
  const int32_t g1 = b.n1[e], g2 = b.n2[e];
  double v1[3], v2[3];
  nd.get(g1, v1);
  nd.get(g2, v2);
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
  const double* w11 = Ws + (size_t)pblk[e * 3 + 0] * 36;
  const double* w12 = Ws + (size_t)pblk[e * 3 + 1] * 36;
  const double* w22 = Ws + (size_t)pblk[e * 3 + 2] * 36;
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
  s += contract_ws(blk, w11, g1, g1, true);
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
  s += contract_ws(blk, w12, g1, g2, false);
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
  s += contract_ws(blk, w22, g2, g2, true);
  if (dir < 6) g_coord[e * 6 + dir] = -s;
  else g_prop[e * 5 + (dir - 6)] = -s;
}

// trusses (3 DOFs per node): directions 0..5 node coordinates, 6 E, 7 A, 8 A2
constexpr int kTrussDirs = 9;
__global__ void __launch_bounds__(128) k_vjp_truss(size_t n_el, NodesView nd, TrussView tv, double abs_tol,
                                                   const double* __restrict__ Ws, const uint32_t* __restrict__ pblk,
                                                   double* __restrict__ g_coord, double* __restrict__ g_prop) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= n_el * kTrussDirs) return;
  const size_t e = t / kTrussDirs;
  const int dir = (int)(t - e * kTrussDirs);
  const int32_t g1 = tv.n1[e], g2 = tv.n2[e];
  double v1[3], v2[3];
  nd.get(g1, v1);
  nd.get(g2, v2);
  Dual x1[3], x2[3], g[9];
  seed3(x1, v1, 0, dir);
  seed3(x2, v2, 3, dir);
  double s = 0.0;
  if (truss_block(x1, x2, Dual(tv.E[e], dir == 6 ? 1.0 : 0.0), Dual(tv.A[e], dir == 7 ? 1.0 : 0.0),
                  Dual(tv.A2[e], dir == 8 ? 1.0 : 0.0), abs_tol, g)) {
    const double* w11 = Ws + (size_t)pblk[e * 3 + 0] * 36;
    const double* w12 = Ws + (size_t)pblk[e * 3 + 1] * 36;
    const double* w22 = Ws + (size_t)pblk[e * 3 + 2] * 36;
    // translational blocks (1,1) = g, (1,2) = (2,1)^T = -g, (2,2) = g; diagonal blocks count Ws at one half
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const double d = g[3 * a + c].d;
        const double w = 0.5 * (w11[6 * a + c] + w22[6 * a + c]) - ws_at(w12, g1, g2, a, c);
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
  // Ws per stiffness block, and the block of every element node pair
  const size_t nb = h->n_blocks;
  CK(h->vjp_Ws.reserve(nb * 36 + 1, s));
  if (nb)
    k_vjp_ws<<<grid_for(nb, kWsBlocksPerCta), 36 * kWsBlocksPerCta, 0, s>>>(nb, h->blk_I.p, h->blk_J.p, h->vjp_lT.p,
                                                                          h->vjp_uT.p, P, h->vjp_Ws.p);
  const size_t pt = h->nt * kPairs2, pb = h->nbm * kPairs2, pp = h->np * kPairs4;
  CK(h->vjp_pblk.reserve(pt + pb + pp + 1, s));
  uint32_t* bt = h->vjp_pblk.p;
  uint32_t* bb = bt + pt;
  uint32_t* bp = bb + pb;
  if (pt) k_pair_blocks<<<grid_for(pt, 256), 256, 0, s>>>(pt, h->slot_t.p, h->blk_start.p, nb, bt);
  if (pb) k_pair_blocks<<<grid_for(pb, 256), 256, 0, s>>>(pb, h->slot_b.p, h->blk_start.p, nb, bb);
  if (pp) k_pair_blocks<<<grid_for(pp, 256), 256, 0, s>>>(pp, h->slot_p.p, h->blk_start.p, nb, bp);
  const size_t ct = h->nt * 6, cb = h->nbm * 6, cp = h->np * 12;
  CK(h->vjp_gc.reserve(ct + cb + cp + 1, s));
  CK(h->vjp_gp.reserve(h->nt * 3 + h->nbm * 5 + h->np * 2 + 1, s));
  const double* Ws = h->vjp_Ws.p;
  double* gct = h->vjp_gc.p;
  double* gcb = gct + ct;
  double* gcp = gcb + cb;
  double* gpt = h->vjp_gp.p;
  double* gpb = gpt + h->nt * 3;
  double* gpp = gpb + h->nbm * 5;
  const NodesView nd = h->nodes();
  if (h->nt)
    k_vjp_truss<<<grid_for(h->nt * kTrussDirs, 128), 128, 0, s>>>(h->nt, nd, h->trusses(), h->abs_tol, Ws, bt, gct,
                                                                   gpt);
  if (h->nbm)
    k_vjp_beam<<<grid_for(h->nbm * kBeamDirs, 128), 128, 0, s>>>(h->nbm, nd, h->beams(), h->rel_tol, h->abs_tol, Ws,
                                                                  bb, gcb, gpb);
  if (h->np)
    k_vjp_plate<<<grid_for(h->np, kPlatesPerCta), kPlateLanes * kPlatesPerCta, 0, s>>>(h->np, nd, h->plates(),
                                                                                       h->abs_tol, Ws, bp, gcp, gpp);
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
  if (!h->pattern_valid) return h->fail(FEM_GPU_ERR_STATE, "call fem_gpu_assemble first");
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
