// fem_loads.cuh -- loads on the nodes (included by fem_gpu.cu, whose handle and
// element arithmetic it uses).
//
// add_concentrated_load, add_uniformly_distributed_line_load and
// add_uniformly_distributed_surface_load (methods_for_bc_data_handle.rs:20-175)
// each add nodal contributions to the forces vector with one `+=` per node, in
// call order.  Here every call appends its contributions (DOF index, value) --
// the element parts computed on the GPU from the element's geometry at the time
// of the call (beam.rs:775-797, plate.rs:1145-1185) -- and the forces vector is
// their ordered sum per DOF: a stable sort by DOF, then one sum per run in call
// order starting from 0, which is the reference's `+=` on a zeroed vector.

// two-node element under a uniformly distributed line load: one Gauss point
// r = 0, alpha = 2, h1 = h2 = 0.5, det J = L / 2; value_i = 0 + (h_i q)(detJ alpha)
__global__ void k_line_loads(size_t n, NodesView nd, const int32_t* __restrict__ bn1, const int32_t* __restrict__ bn2,
                             const int32_t* __restrict__ elem, const uint8_t* __restrict__ dof,
                             const double* __restrict__ q, unsigned long long* __restrict__ key,
                             double* __restrict__ val) {
  const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int32_t b = elem[k], a = bn1[b], c = bn2[b];
  double x1[3], x2[3], d[3];
  nd.get(a, x1);
  nd.get(c, x2);
  sub3(x2, x1, d);
  const double jac = norm3(d) * 0.5;
  const double h1 = 0.5 * (1.0 - 0.0), h2 = 0.5 * (1.0 + 0.0);
  key[2 * k] = 6ull * (unsigned long long)a + dof[k];
  val[2 * k] = 0.0 + (h1 * q[k]) * (jac * 2.0);
  key[2 * k + 1] = 6ull * (unsigned long long)c + dof[k];
  val[2 * k + 1] = 0.0 + (h2 * q[k]) * (jac * 2.0);
}

// plate under a uniformly distributed surface load: 2 x 2 Gauss points in the
// stiffness's order, alpha_r = alpha_s = 1, h_i(r, s) = (0.25 (1 +- r))(1 +- s),
// det J(r, s) = det(4 J) / 16 from the local coordinates, exactly as the
// stiffness computes it; value_i = sum over the points, in order, from 0
__global__ void k_surface_loads(size_t n, NodesView nd, PlateView pl, double abs_tol, const int32_t* __restrict__ elem,
                                const uint8_t* __restrict__ dof, const double* __restrict__ q,
                                unsigned long long* __restrict__ key, double* __restrict__ val) {
  const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int32_t p = elem[k];
  const int32_t nidx[4] = {pl.n1[p], pl.n2[p], pl.n3[p], pl.n4[p]};
  double X[4][3];
#pragma unroll
  for (int i = 0; i < 4; ++i) nd.get(nidx[i], X[i]);
  double R[9];
  if (!plate_rotation(X[1], X[2], X[3], abs_tol, R)) set_identity(R);
  double xl[4] = {0.0, 0.0, 0.0, 0.0}, yl[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    if (i == 2) continue;
    double dd[3];
    sub3(X[i], X[2], dd);
    xl[i] = (R[0] * dd[0] + R[1] * dd[1]) + R[2] * dd[2];
    yl[i] = (R[3] * dd[0] + R[4] * dd[1]) + R[5] * dd[2];
  }
  const double g = sqrt((double)(1.0f / 3.0f));
  const double ipr[4] = {g * 1.0, g * -1.0, g * -1.0, g * 1.0};
  const double ips[4] = {g * 1.0, g * 1.0, g * -1.0, g * -1.0};
  const double d12x = xl[0] - xl[1], d12y = yl[0] - yl[1];
  const double ax = d12x + xl[3], bx = d12x - xl[3], cx = (xl[0] + xl[1]) - xl[3];
  const double ay = d12y + yl[3], by = d12y - yl[3], cy = (yl[0] + yl[1]) - yl[3];
  double out[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
  for (int ip = 0; ip < 4; ++ip) {
    const double r = ipr[ip], s = ips[ip];
    const double J00 = fma(s, bx, ax), J01 = fma(s, by, ay), J10 = fma(r, bx, cx), J11 = fma(r, by, cy);
    const double detj = fma(J00, J11, -(J01 * J10)) * 0.0625;
    const double w = (detj * 1.0) * 1.0;
    const double h[4] = {(0.25 * (1.0 + r)) * (1.0 + s), (0.25 * (1.0 - r)) * (1.0 + s),
                         (0.25 * (1.0 - r)) * (1.0 - s), (0.25 * (1.0 + r)) * (1.0 - s)};
#pragma unroll
    for (int i = 0; i < 4; ++i) out[i] = out[i] + (h[i] * q[k]) * w;
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    key[4 * k + i] = 6ull * (unsigned long long)nidx[i] + dof[k];
    val[4 * k + i] = out[i];
  }
}

__global__ void k_iota(size_t n, uint32_t* __restrict__ out) {
  const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k < n) out[k] = (uint32_t)k;
}

// the forces vector: every run of equal DOFs in the stably sorted contributions, summed in call order from 0
__global__ void k_force_runs(size_t n, const unsigned long long* __restrict__ skey, const uint32_t* __restrict__ sidx,
                             const double* __restrict__ val, double* __restrict__ forces) {
  const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k >= n || (k > 0 && skey[k - 1] == skey[k])) return;
  double acc = 0.0;
  size_t j = k;
  do {
    acc = acc + val[sidx[j]];
    ++j;
  } while (j < n && skey[j] == skey[k]);
  forces[skey[k]] = acc;
}

namespace {

// room for m more contributions after the n_ld already stored
int loads_reserve(fem_gpu* h, size_t m) {
  CK(h->ld_key.reserve(h->n_ld + m + 1, h->stream, h->n_ld));
  CK(h->ld_val.reserve(h->n_ld + m + 1, h->stream, h->n_ld));
  return FEM_GPU_OK;
}

// element loads: look the elements up (stopping at the first that does not exist), then compute their
// contributions on the GPU
int element_loads(fem_gpu* h, bool plates, const uint32_t* numbers, const uint8_t* dofs, const double* values,
                  size_t n, size_t* n_added) {
  if (n_added) *n_added = 0;
  if (!h || (n && (!numbers || !dofs || !values))) return FEM_GPU_ERR_ARGUMENT;
  int st = ensure_ready(h);
  if (st) return st;
  HostVec<int32_t> idx(n);
  size_t k = 0;
  int code = FEM_GPU_OK;
  for (; k < n; ++k) {
    if (dofs[k] > 5) {
      code = h->fail(FEM_GPU_ERR_ARGUMENT, "Incorrect dof parameter number!");
      break;
    }
    const int64_t e = plates ? h->p_by_num.find(numbers[k]) : h->b_by_num.find(numbers[k]);
    if (e < 0) {
      code = h->fail(FEM_GPU_ERR_ELEM_NOT_EXIST, plates ? "Plate element with number %u does not exist!"
                                                        : "Beam element with number %u does not exist!",
                     numbers[k]);
      break;
    }
    idx[k] = (int32_t)e;
  }
  if (k) {
    const size_t per = plates ? 4 : 2;
    st = loads_reserve(h, per * k);
    if (st) return st;
    DevBuf<int32_t> d_idx;
    DevBuf<uint8_t> d_dof;
    DevBuf<double> d_q;
    CK(upload(d_idx, 0, idx.data(), k, h->stream));
    CK(upload(d_dof, 0, dofs, k, h->stream));
    CK(upload(d_q, 0, values, k, h->stream));
    unsigned long long* key = h->ld_key.p + h->n_ld;
    double* val = h->ld_val.p + h->n_ld;
    if (plates)
      k_surface_loads<<<grid_for(k, 128), 128, 0, h->stream>>>(k, h->nodes(), h->plates(), h->abs_tol, d_idx.p,
                                                               d_dof.p, d_q.p, key, val);
    else
      k_line_loads<<<grid_for(k, 128), 128, 0, h->stream>>>(k, h->nodes(), h->b_n1.p, h->b_n2.p, d_idx.p, d_dof.p,
                                                            d_q.p, key, val);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->stream));
    h->n_ld += per * k;
    h->forces_valid = false;
  }
  if (n_added) *n_added = k;
  return code;
}

}  // namespace

extern "C" int fem_gpu_add_concentrated_loads(fem_gpu_t* h, const uint32_t* node_numbers, const uint8_t* dofs,
                                              const double* values, size_t n, size_t* n_added) {
  if (n_added) *n_added = 0;
  if (!h || (n && (!node_numbers || !dofs || !values))) return FEM_GPU_ERR_ARGUMENT;
  int st = ensure_ready(h);
  if (st) return st;
  HostVec<unsigned long long> key(n);
  size_t k = 0;
  int code = FEM_GPU_OK;
  for (; k < n; ++k) {
    if (dofs[k] > 5) {
      code = h->fail(FEM_GPU_ERR_ARGUMENT, "Incorrect dof parameter number!");
      break;
    }
    int32_t i = 0;
    if ((code = lookup_node(h, node_numbers[k], &i))) break;
    key[k] = 6ull * (unsigned long long)i + dofs[k];
  }
  if (k) {
    st = loads_reserve(h, k);
    if (st) return st;
    CK(cudaMemcpyAsync(h->ld_key.p + h->n_ld, key.data(), k * sizeof(unsigned long long), cudaMemcpyHostToDevice,
                       h->stream));
    CK(cudaMemcpyAsync(h->ld_val.p + h->n_ld, values, k * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    h->n_ld += k;
    h->forces_valid = false;
  }
  if (n_added) *n_added = k;
  return code;
}

extern "C" int fem_gpu_add_line_loads(fem_gpu_t* h, const uint32_t* beam_numbers, const uint8_t* dofs,
                                      const double* values, size_t n, size_t* n_added) {
  return element_loads(h, false, beam_numbers, dofs, values, n, n_added);
}

extern "C" int fem_gpu_add_surface_loads(fem_gpu_t* h, const uint32_t* plate_numbers, const uint8_t* dofs,
                                         const double* values, size_t n, size_t* n_added) {
  return element_loads(h, true, plate_numbers, dofs, values, n, n_added);
}

namespace {
int forces_update(fem_gpu* h) {
  if (h->forces_valid) return FEM_GPU_OK;
  cudaStream_t s = h->stream;
  const size_t nd = (size_t)h->nodes_number * 6, n = h->n_ld;
  CK(h->forces.reserve(nd + 1, s));
  if (nd) CK(cudaMemsetAsync(h->forces.p, 0, nd * sizeof(double), s));
  if (n) {
    DevBuf<unsigned long long> skey;
    DevBuf<uint32_t> idx, sidx;
    CK(skey.reserve(n, s));
    CK(idx.reserve(n, s));
    CK(sidx.reserve(n, s));
    k_iota<<<grid_for(n, 256), 256, 0, s>>>(n, idx.p);
    int end_bit = 1;
    while (end_bit < 64 && (nd >> end_bit)) ++end_bit;
    int st = cub_call(h, [&](void* tmp, size_t& bytes) {
      return cub::DeviceRadixSort::SortPairs(tmp, bytes, h->ld_key.p, skey.p, idx.p, sidx.p, (int64_t)n, 0, end_bit,
                                             s);
    });
    if (st) return st;
    k_force_runs<<<grid_for(n, 256), 256, 0, s>>>(n, skey.p, sidx.p, h->ld_val.p, h->forces.p);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s));
  }
  h->forces_valid = true;
  return FEM_GPU_OK;
}
}  // namespace

extern "C" int fem_gpu_get_forces(fem_gpu_t* h, double* forces) {
  if (!h || !forces) return FEM_GPU_ERR_ARGUMENT;
  int st = ensure_ready(h);
  if (st) return st;
  st = forces_update(h);
  if (st) return st;
  const size_t nd = (size_t)h->nodes_number * 6;
  if (nd) CK(cudaMemcpyAsync(forces, h->forces.p, nd * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_get_forces_device(fem_gpu_t* h, const double** forces) {
  if (!h || !forces) return FEM_GPU_ERR_ARGUMENT;
  int st = ensure_ready(h);
  if (st) return st;
  st = forces_update(h);
  if (st) return st;
  *forces = h->forces.p;
  return FEM_GPU_OK;
}
