// fem_results.cuh -- element results (included by fem_gpu.cu, whose handle and
// element arithmetic it uses).
//
// extract_elements_analysis_result (methods_for_element_analysis.rs:27-58)
// turns the displacements vector into per-element forces and moments:
// truss.rs:281-333 (ForceR), beam.rs:803-993 (ForceR, ForceS, ForceT, MomentR,
// MomentS and MomentT at node 1 / mid-length / node 2) and plate.rs:1196-1409
// (membrane forces, bending moments and transverse shear forces summed over
// the four corner points).  One thread per element: the element's node
// coordinates and displacements (48 bytes per node, read as three 16-byte
// loads) are gathered, the rotation is recomputed exactly as the stiffness
// computes it, and the results are written as 16-byte stores.  The arithmetic
// is FP64-bound (a few hundred operations per plate against ~150 bytes of
// traffic), so the kernels are plain one-element-per-thread grids sized to the
// element count.  Every expression below follows the oracle's restatement
// operation by operation (the GPU is built with --fmad=false).

namespace {

__device__ __forceinline__ double res_row(const double R[9], int i, const double u[3]) {
  return fma(R[3 * i + 2], u[2], fma(R[3 * i + 1], u[1], R[3 * i] * u[0]));
}

// the six displacements of node i (index order, 6 per node)
__device__ __forceinline__ void res_node_u(const double* __restrict__ disp, int32_t i, double u[6]) {
  const double2* p = reinterpret_cast<const double2*>(disp + 6 * (size_t)i);
  const double2 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
  u[0] = a.x;
  u[1] = a.y;
  u[2] = b.x;
  u[3] = b.y;
  u[4] = c.x;
  u[5] = c.y;
}

}  // namespace

// truss: strain (u2 - u1) / L on the local axial displacements, ForceR = strain (E area)
__global__ void __launch_bounds__(256) k_truss_results(size_t n, NodesView nd, TrussView t, double abs_tol,
                                                       const double* __restrict__ disp, double* __restrict__ out) {
  const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= n) return;
  const int32_t I = t.n1[e], J = t.n2[e];
  double x1[3], x2[3], R[9];
  nd.get(I, x1);
  nd.get(J, x2);
  if (!truss_rotation(x1, x2, abs_tol, R)) {
    out[e] = __longlong_as_double(0x7ff8000000000000ll);
    return;
  }
  double d[3];
  sub3(x2, x1, d);
  const double L = norm3(d);
  const double A = t.A[e], A2 = t.A2[e];
  double a_r = A;
  if (A2 == A2) a_r = A + (A2 - A) * 0.5;
  const double* p1 = disp + 6 * (size_t)I;
  const double* p2 = disp + 6 * (size_t)J;
  const double2 a = __ldg(reinterpret_cast<const double2*>(p1)), b = __ldg(reinterpret_cast<const double2*>(p2));
  const double u1v[3] = {a.x, a.y, __ldg(p1 + 2)}, u2v[3] = {b.x, b.y, __ldg(p2 + 2)};
  const double u1 = res_row(R, 0, u1v), u2 = res_row(R, 0, u2v);
  out[e] = ((u2 - u1) * (1.0 / L)) * (t.E[e] * a_r);
}

// beam: the six strains of the one-point rule on the local displacements; out 10 per beam
__global__ void __launch_bounds__(256) k_beam_results(size_t n, NodesView nd, BeamView b, double rel_tol,
                                                      double abs_tol, const double* __restrict__ disp,
                                                      double* __restrict__ out) {
  const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= n) return;
  const int32_t I = b.n1[e], J = b.n2[e];
  double x1[3], x2[3], R[9], i11p, i22p;
  nd.get(I, x1);
  nd.get(J, x2);
  const double axis[3] = {b.ax[e], b.ay[e], b.az[e]};
  double2* o = reinterpret_cast<double2*>(out + 10 * e);
  if (!beam_rotation(x1, x2, b.i11[e], b.i22[e], b.i12[e], axis, rel_tol, abs_tol, R, i11p, i22p)) {
    const double q = __longlong_as_double(0x7ff8000000000000ll);
#pragma unroll
    for (int k = 0; k < 5; ++k) o[k] = make_double2(q, q);
    return;
  }
  double d[3];
  sub3(x2, x1, d);
  const double L = norm3(d);
  const double s = 1.0 / L;
  double u[12], ul[12];
  res_node_u(disp, I, u);
  res_node_u(disp, J, u + 6);
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int i = 0; i < 3; ++i) ul[3 * k + i] = res_row(R, i, u + 3 * k);
  const double E = b.E[e], A = b.A[e];
  const double G = E / (2.0 * (1.0 + b.nu[e]));
  const double gak = (G * A) * b.ks[e];
  const double eu = (ul[6] - ul[0]) * s;
  const double ev = fma(ul[7] - ul[1], s, (ul[5] + ul[11]) * -0.5);
  const double ew = fma(ul[8] - ul[2], s, (ul[4] + ul[10]) * -0.5);
  const double fr = eu * (E * A);
  const double fs = ev * gak;
  const double ft = ew * gak;
  const double mr = ((ul[9] - ul[3]) * s) * (G * b.it[e]);
  const double ms = ((ul[10] - ul[4]) * s) * (E * i22p);
  const double mt = ((ul[11] - ul[5]) * s) * (E * i11p);
  const double hs = (L * ft) * 0.5, ht = (L * fs) * 0.5;
  o[0] = make_double2(fr, fs);
  o[1] = make_double2(ft, mr);
  o[2] = make_double2(ms + hs, ms);
  o[3] = make_double2(ms - hs, mt + ht);
  o[4] = make_double2(mt, mt - ht);
}

// plate: the corner-point strain sums as weighted sums of the nodal fields' differences along the four edges
// (1-2, 4-3 along r, 1-4, 2-3 along s; corner k spans one r and one s edge, d_k = r edge x s edge = 4 det J),
// one shared reciprocal for the four corner determinants; out 8 per plate
__global__ void __launch_bounds__(256) k_plate_results(size_t n, NodesView nd, PlateView pl, double abs_tol,
                                                       const double* __restrict__ disp, double* __restrict__ out) {
  const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= n) return;
  const int32_t nidx[4] = {pl.n1[e], pl.n2[e], pl.n3[e], pl.n4[e]};
  double X[4][3];
#pragma unroll
  for (int i = 0; i < 4; ++i) nd.get(nidx[i], X[i]);
  double2* o = reinterpret_cast<double2*>(out + 8 * e);
  double R[9];
  if (!plate_rotation(X[1], X[2], X[3], abs_tol, R)) {
    const double q = __longlong_as_double(0x7ff8000000000000ll);
#pragma unroll
    for (int k = 0; k < 4; ++k) o[k] = make_double2(q, q);
    return;
  }
  double xl[4] = {0.0, 0.0, 0.0, 0.0}, yl[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    if (i == 2) continue;
    double dd[3];
    sub3(X[i], X[2], dd);
    xl[i] = (R[0] * dd[0] + R[1] * dd[1]) + R[2] * dd[2];
    yl[i] = (R[3] * dd[0] + R[4] * dd[1]) + R[5] * dd[2];
  }
  double fu[4], fv[4], fw[4], ftx[4], fty[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    double u[6];
    res_node_u(disp, nidx[i], u);
    fu[i] = res_row(R, 0, u);
    fv[i] = res_row(R, 1, u);
    fw[i] = res_row(R, 2, u);
    ftx[i] = res_row(R, 0, u + 3);
    fty[i] = res_row(R, 1, u + 3);
  }
  constexpr int eh[4] = {0, 3, 0, 1}, et[4] = {1, 2, 3, 2};
  double ex[4], ey[4], el[4], Fu[4], Fv[4], Ftx[4], Fty[4], Gm[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int p = eh[k], q = et[k];
    ex[k] = xl[p] - xl[q];
    ey[k] = yl[p] - yl[q];
    el[k] = sqrt(fma(ex[k], ex[k], ey[k] * ey[k]));
    Fu[k] = fu[p] - fu[q];
    Fv[k] = fv[p] - fv[q];
    Ftx[k] = ftx[p] - ftx[q];
    Fty[k] = fty[p] - fty[q];
    Gm[k] = fma(fma(ex[k], fty[p] + fty[q], -(ey[k] * (ftx[p] + ftx[q]))), 0.5, fw[p] - fw[q]);
  }
  double dk[4];
  dk[0] = fma(ex[0], ey[2], -(ey[0] * ex[2]));
  dk[1] = fma(ex[0], ey[3], -(ey[0] * ex[3]));
  dk[2] = fma(ex[1], ey[3], -(ey[1] * ex[3]));
  dk[3] = fma(ex[1], ey[2], -(ey[1] * ex[2]));
  double q[4];
  {
    const double d01 = dk[0] * dk[1], d23 = dk[2] * dk[3];
    const double inv = 1.0 / (d01 * d23);
    q[0] = (dk[1] * d23) * inv;
    q[1] = (dk[0] * d23) * inv;
    q[2] = (dk[3] * d01) * inv;
    q[3] = (dk[2] * d01) * inv;
  }
  // edge weights of the corner sums of d/dx and d/dy
  const double Wx[4] = {fma(ey[2], q[0], ey[3] * q[1]), fma(ey[3], q[2], ey[2] * q[3]),
                        -fma(ey[0], q[0], ey[1] * q[3]), -fma(ey[0], q[1], ey[1] * q[2])};
  const double Wy[4] = {-fma(ex[2], q[0], ex[3] * q[1]), -fma(ex[3], q[2], ex[2] * q[3]),
                        fma(ex[0], q[0], ex[1] * q[3]), fma(ex[0], q[1], ex[1] * q[2])};
  double e0 = Wx[0] * Fu[0], e1 = Wy[0] * Fv[0], k0 = Wx[0] * Fty[0], k1 = Wy[0] * Ftx[0];
  double e2 = fma(Wx[0], Fv[0], Wy[0] * Fu[0]), k2 = fma(Wx[0], Ftx[0], -(Wy[0] * Fty[0]));
#pragma unroll
  for (int k = 1; k < 4; ++k) {
    e0 = fma(Wx[k], Fu[k], e0);
    e1 = fma(Wy[k], Fv[k], e1);
    e2 = fma(Wx[k], Fv[k], fma(Wy[k], Fu[k], e2));
    k0 = fma(Wx[k], Fty[k], k0);
    k1 = fma(Wy[k], Ftx[k], k1);
    k2 = fma(-Wy[k], Fty[k], fma(Wx[k], Ftx[k], k2));
  }
  k0 = -k0;
  const double g0 = fma(Gm[1], fma(el[3], q[2], el[2] * q[3]), Gm[0] * fma(el[2], q[0], el[3] * q[1]));
  const double g1 = fma(Gm[3], fma(el[0], q[1], el[1] * q[2]), Gm[2] * fma(el[0], q[0], el[1] * q[3]));
  const double young = pl.E[e], nu = pl.nu[e], t = pl.t[e];
  // one division: E / (2 (1 + nu)) = E ((1 - nu) / 2) / (1 - nu^2), and t^2 / 24 by the constant 1/24
  const double dinv = 1.0 / (1.0 - nu * nu);
  const double hn = (1.0 - nu) * 0.5;
  const double cm = (young * dinv) * (t * 0.25);
  const double cbm = ((young * t) * (0.5 * dinv)) * ((t * t) * (1.0 / 24.0));
  const double cs = ((young * hn) * dinv) * ((t * pl.ks[e]) * 0.25);
  o[0] = make_double2(cm * fma(nu, e1, e0), cm * fma(nu, e0, e1));
  o[1] = make_double2(cm * (hn * e2), cbm * fma(nu, k0, k1));
  o[2] = make_double2(cbm * fma(nu, k1, k0), cbm * (hn * k2));
  o[3] = make_double2(cs * g0, cs * g1);
}

namespace {

// the three result kernels on the handle's stream, bracketed by the handle's events
int results_launch(fem_gpu* h, const double* disp, double* t_out, double* b_out, double* p_out) {
  cudaStream_t s = h->stream;
  NodesView nd = h->nodes();
  for (auto& ev : h->res_ev)
    if (!ev) CK(cudaEventCreate(&ev));
  CK(cudaEventRecord(h->res_ev[0], s));
  if (t_out && h->nt)
    k_truss_results<<<grid_for(h->nt, 256), 256, 0, s>>>(h->nt, nd, h->trusses(), h->abs_tol, disp, t_out);
  if (b_out && h->nbm)
    k_beam_results<<<grid_for(h->nbm, 256), 256, 0, s>>>(h->nbm, nd, h->beams(), h->rel_tol, h->abs_tol, disp,
                                                          b_out);
  if (p_out && h->np)
    k_plate_results<<<grid_for(h->np, 256), 256, 0, s>>>(h->np, nd, h->plates(), h->abs_tol, disp, p_out);
  CK(cudaGetLastError());
  CK(cudaEventRecord(h->res_ev[1], s));
  h->res_timed = true;
  return FEM_GPU_OK;
}

bool misaligned16(const void* p) { return ((uintptr_t)p & 15u) != 0; }

}  // namespace

extern "C" int fem_gpu_element_results(fem_gpu_t* h, const double* displacements, size_t n_displacements,
                                       double* truss_out, double* beam_out, double* plate_out) {
  if (!h || !displacements) return FEM_GPU_ERR_ARGUMENT;
  int st = ensure_ready(h);
  if (st) return st;
  if (n_displacements < 6 * h->n_nodes)
    return h->fail(FEM_GPU_ERR_ARGUMENT, "the displacements vector has %zu entries, the model %zu nodes",
                   n_displacements, h->n_nodes);
  cudaStream_t s = h->stream;
  const size_t nd6 = 6 * h->n_nodes;
  const size_t nt = truss_out ? h->nt : 0, nb = beam_out ? h->nbm : 0, np = plate_out ? h->np : 0;
  // device layout: displacements, then beam (10 per), plate (8 per) and truss (1 per) results; every part
  // starts on a 16-byte boundary (all sizes are even but the truss part, which is last)
  const size_t ob = nd6, op = ob + 10 * nb, ot = op + 8 * np;
  CK(h->res_buf.reserve(ot + nt + 2, s));
  double* base = h->res_buf.p;
  if (nd6) CK(cudaMemcpyAsync(base, displacements, nd6 * sizeof(double), cudaMemcpyHostToDevice, s));
  st = results_launch(h, base, nt ? base + ot : nullptr, nb ? base + ob : nullptr, np ? base + op : nullptr);
  if (st) return st;
  if (nb) CK(cudaMemcpyAsync(beam_out, base + ob, 10 * nb * sizeof(double), cudaMemcpyDeviceToHost, s));
  if (np) CK(cudaMemcpyAsync(plate_out, base + op, 8 * np * sizeof(double), cudaMemcpyDeviceToHost, s));
  if (nt) CK(cudaMemcpyAsync(truss_out, base + ot, nt * sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_element_results_device(fem_gpu_t* h, const double* displacements, double* truss_out,
                                              double* beam_out, double* plate_out) {
  if (!h || !displacements) return FEM_GPU_ERR_ARGUMENT;
  if (misaligned16(displacements) || misaligned16(beam_out) || misaligned16(plate_out))
    return h->fail(FEM_GPU_ERR_ARGUMENT, "device arrays must start on a 16-byte boundary");
  int st = ensure_ready(h);
  if (st) return st;
  return results_launch(h, displacements, truss_out, beam_out, plate_out);
}

extern "C" int fem_gpu_results_last_ms(fem_gpu_t* h, float* ms) {
  if (!h || !ms) return FEM_GPU_ERR_ARGUMENT;
  if (!h->res_timed) return h->fail(FEM_GPU_ERR_STATE, "no element results computed yet");
  CK(cudaEventSynchronize(h->res_ev[1]));
  CK(cudaEventElapsedTime(ms, h->res_ev[0], h->res_ev[1]));
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_get_element_numbers(fem_gpu_t* h, int kind, uint32_t* numbers) {
  if (!h || !numbers || kind < 0 || kind > 2) return FEM_GPU_ERR_ARGUMENT;
  const HostVec<uint32_t>& v = kind == 0 ? h->t_num : kind == 1 ? h->b_num : h->p_num;
  if (!v.empty()) memcpy(numbers, v.data(), v.size() * sizeof(uint32_t));
  return FEM_GPU_OK;
}
