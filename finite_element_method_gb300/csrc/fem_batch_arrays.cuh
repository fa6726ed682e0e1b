// fem_batch_arrays.cuh -- a batch built from the host arrays of many
// structures (included by fem_gpu.cu after fem_batch.cuh, whose batch object,
// graph and autotuner it reuses).
//
// fem_gpu_batch_create_from_arrays stands for one plain call sequence per
// structure -- FEM::create(rel_tol, abs_tol, nodes_number[i]), add_nodes of its
// nodes, add_trusses, add_beams and add_plates of its elements, assemble --
// done for every structure at once:
//
//   * the checks of all structures run as bulk GPU passes over all items:
//     radix sorts of (structure, number) keys find repeated node and element
//     numbers, sorted hashes with exact comparison find repeated coordinates
//     and plate node sets, sorted node pairs find repeated two-node elements,
//     a binary search of (structure, node number) finds every element node,
//     and the validation kernels of the plain path check every element;
//   * the structures are laid side by side as one union model: structure i
//     owns the node slots [cap_off[i], cap_off[i] + nodes_number[i]) and so the
//     stiffness rows [6 cap_off[i], 6 cap_off[i + 1]);
//   * one symbolic phase builds the union's pattern, and the numeric pass of
//     every structure is one CUDA-graph launch (persistent or plain element
//     launches, as the autotuner picks, then the block sums and the gather).
//
// Node-pair blocks never span structures and each structure keeps its call
// order (its trusses, then its beams, then its plates, each in input order), so
// every value is bit-identical to the structure's own plain assembly.  The
// columns of every structure are stored relative to its first node slot, and
// its row starts relative to its first entry: structure i's CSR is exactly the
// one its plain assembly gives.
//
// A structure flagged by the bulk checks is replayed through the plain calls,
// which give the error code and message of its first failing call; the batch
// then fails with that error (prefixed by the structure's index).  The bulk
// checks can flag a valid structure (two different items with equal hashes in
// a group of three or more), never miss an invalid one: a replay that
// succeeds just moves on to the next flagged structure.

namespace {

// the structure of item i: off[s] <= i < off[s + 1] (off is nondecreasing, off[0] = 0)
__global__ void k_ba_sid(const unsigned long long* __restrict__ off, uint32_t n_struct, size_t n,
                         uint32_t* __restrict__ sid) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t lo = 0, hi = n_struct;  // invariant: off[lo] <= i < off[hi]
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (off[mid] <= i) lo = mid;
    else hi = mid;
  }
  sid[i] = lo;
}

// (structure, number) keys of nodes or elements
__global__ void k_ba_num_keys(size_t n, const uint32_t* __restrict__ sid, const uint32_t* __restrict__ num,
                              unsigned long long* __restrict__ key, uint32_t* __restrict__ idx) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  key[i] = ((unsigned long long)sid[i] << 32) | num[i];
  idx[i] = (uint32_t)i;
}

// equal neighbouring keys: the structure of the later item fails
__global__ void k_ba_equal_keys(size_t n, const unsigned long long* __restrict__ skey,
                                const uint32_t* __restrict__ sidx, const uint32_t* __restrict__ sid,
                                int* __restrict__ fail) {
  const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k == 0 || k >= n || skey[k] == kNoKey || skey[k] != skey[k - 1]) return;
  fail[sid[sidx[k]]] = 1;
}

// coordinate keys: the plain path's hash of the exact coordinates (-0.0 as 0.0, NaN equal to nothing),
// mixed with the structure
__global__ void k_ba_coord_keys(size_t n, const uint32_t* __restrict__ sid, const double* __restrict__ xyz,
                                unsigned long long* __restrict__ key, uint32_t* __restrict__ idx) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double a = xyz[3 * i], b = xyz[3 * i + 1], c = xyz[3 * i + 2];
  idx[i] = (uint32_t)i;
  if (a != a || b != b || c != c) {
    key[i] = kNoKey;
    return;
  }
  if (a == 0.0) a = 0.0;
  if (b == 0.0) b = 0.0;
  if (c == 0.0) c = 0.0;
  const unsigned long long ha = (unsigned long long)__double_as_longlong(a),
                           hb = (unsigned long long)__double_as_longlong(b),
                           hc = (unsigned long long)__double_as_longlong(c);
  key[i] = dev_mix64(ha ^ dev_mix64(hb ^ dev_mix64(hc ^ dev_mix64(0x9e3779b97f4a7c15ull + sid[i])))) >> 1;
}

// inside a group of equal coordinate keys: an item equal to an earlier one of its structure fails it
__global__ void k_ba_coord_dups(size_t n, const unsigned long long* __restrict__ skey,
                                const uint32_t* __restrict__ sidx, const uint32_t* __restrict__ sid,
                                const double* __restrict__ xyz, int* __restrict__ fail) {
  const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k == 0 || k >= n || skey[k] == kNoKey || skey[k - 1] != skey[k]) return;
  const uint32_t j = sidx[k];
  const double* a = xyz + 3 * (size_t)j;
  for (size_t p = k; p-- > 0 && skey[p] == skey[k];) {
    const uint32_t i = sidx[p];
    const double* b = xyz + 3 * (size_t)i;
    if (sid[i] == sid[j] && a[0] == b[0] && a[1] == b[1] && a[2] == b[2]) {
      fail[sid[j]] = 1;
      return;
    }
  }
}

// node slot of every element node: (structure, node number) searched among the sorted node keys;
// a number the structure does not have fails it (and points at the structure's first slot)
__global__ void k_ba_lookup(size_t n, int per_el, const uint32_t* __restrict__ el_sid,
                            const uint32_t* __restrict__ el_nodes, const unsigned long long* __restrict__ nkey,
                            const uint32_t* __restrict__ nidx, size_t n_nodes, const unsigned long long* __restrict__ node_off,
                            const unsigned long long* __restrict__ cap_off, int32_t* out0, int32_t* out1, int32_t* out2,
                            int32_t* out3, int* __restrict__ fail) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= n * per_el) return;
  const size_t e = t / per_el;
  const int c = (int)(t - e * per_el);
  const uint32_t s = el_sid[e];
  const unsigned long long want = ((unsigned long long)s << 32) | el_nodes[t];
  size_t lo = 0, hi = n_nodes;  // first position with nkey >= want
  while (lo < hi) {
    const size_t mid = (lo + hi) >> 1;
    if (nkey[mid] < want) lo = mid + 1;
    else hi = mid;
  }
  int32_t slot = (int32_t)cap_off[s];
  const bool found = lo < n_nodes && nkey[lo] == want;
  const unsigned long long local = found ? nidx[lo] - node_off[s] : 0ull;
  if (found && cap_off[s] + local < cap_off[s + 1]) slot = (int32_t)(cap_off[s] + local);
  else fail[s] = 1;  // no such node, or a node past the structure's room (the structure fails anyway)
  int32_t* out = c == 0 ? out0 : c == 1 ? out1 : c == 2 ? out2 : out3;
  out[e] = slot;
}

// coordinates into their structure's node slots
__global__ void k_ba_place_nodes(size_t n, const uint32_t* __restrict__ sid, const double* __restrict__ xyz,
                                 const unsigned long long* __restrict__ node_off,
                                 const unsigned long long* __restrict__ cap_off, double* x, double* y, double* z) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t s = sid[i];
  const size_t slot = cap_off[s] + (i - node_off[s]);
  if (slot >= cap_off[s + 1]) return;  // more nodes than room: the structure fails
  x[slot] = xyz[3 * i];
  y[slot] = xyz[3 * i + 1];
  z[slot] = xyz[3 * i + 2];
}

// two-node elements: the node-slot pair (slots are distinct across structures)
__global__ void k_ba_pair_keys(size_t n, const int32_t* __restrict__ n1, const int32_t* __restrict__ n2,
                               unsigned long long* __restrict__ key, uint32_t* __restrict__ idx) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t a = (uint32_t)n1[i], b = (uint32_t)n2[i];
  key[i] = a < b ? ((unsigned long long)a << 32 | b) : ((unsigned long long)b << 32 | a);
  idx[i] = (uint32_t)i;
}

// plates: equal sorted slot sets inside a group of equal hashes fail the later plate's structure
__global__ void k_ba_set4_dups(size_t n, const unsigned long long* __restrict__ skey, const uint32_t* __restrict__ sidx,
                               const int32_t* __restrict__ n1, const int32_t* __restrict__ n2,
                               const int32_t* __restrict__ n3, const int32_t* __restrict__ n4,
                               const uint32_t* __restrict__ sid, int* __restrict__ fail) {
  const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k == 0 || k >= n || skey[k - 1] != skey[k]) return;
  const uint32_t j = sidx[k];
  const uint4 v = dev_sorted4(n1[j], n2[j], n3[j], n4[j]);
  for (size_t p = k; p-- > 0 && skey[p] == skey[k];) {
    const uint32_t i = sidx[p];
    const uint4 w = dev_sorted4(n1[i], n2[i], n3[i], n4[i]);
    if (w.x == v.x && w.y == v.y && w.z == v.z && w.w == v.w) {
      fail[sid[j]] = 1;
      return;
    }
  }
}

__global__ void k_ba_status(size_t n, const int* __restrict__ status, const uint32_t* __restrict__ sid,
                            int* __restrict__ fail) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n && status[i]) fail[sid[i]] = 1;
}

__global__ void k_ba_split3(size_t n, const double* __restrict__ v3, double* a, double* b, double* c) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  a[i] = v3[3 * i];
  b[i] = v3[3 * i + 1];
  c[i] = v3[3 * i + 2];
}

__global__ void k_ba_fill(size_t n, double v, double* a) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) a[i] = v;
}

// after the symbolic phase: every structure's columns relative to its first node slot, its row starts
// relative to its first entry (rows of structure s: [6 cap_off[s], 6 cap_off[s + 1]))
__global__ void k_ba_localise(size_t n_rows, const unsigned long long* __restrict__ cap_off, uint32_t n_struct,
                              const int64_t* __restrict__ row_ptr, int32_t* __restrict__ col_idx,
                              int64_t* __restrict__ row_local) {
  const size_t r = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (r >= n_rows) return;
  const size_t node = r / 6;
  uint32_t lo = 0, hi = n_struct;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (cap_off[mid] <= node) lo = mid;
    else hi = mid;
  }
  const int64_t base = row_ptr[6 * cap_off[lo]];
  const int32_t c0 = (int32_t)(6 * cap_off[lo]);
  row_local[r] = row_ptr[r] - base;
  for (int64_t k = row_ptr[r]; k < row_ptr[r + 1]; ++k) col_idx[k] -= c0;
}

// the first CSR entry of every structure (and the total after the last)
__global__ void k_ba_entry_offsets(size_t n, const unsigned long long* __restrict__ cap_off,
                                   const int64_t* __restrict__ row_ptr, int64_t* __restrict__ out) {
  const size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (q < n) out[q] = row_ptr[6 * cap_off[q]];
}

// one structure through the plain calls: the first failing call's status and message
int ba_replay(double rel_tol, double abs_tol, const fem_gpu_structures_t* in, size_t s, std::string* msg) {
  fem_gpu_t* h = nullptr;
  int st = fem_gpu_create(rel_tol, abs_tol, in->nodes_number[s], &h);
  if (st) return st;
  size_t n = 0;
  const size_t n0 = in->node_off[s], nn = in->node_off[s + 1] - n0;
  st = fem_gpu_add_nodes(h, in->node_numbers + n0, in->xyz + 3 * n0, nn, &n);
  const size_t t0 = in->truss_off ? in->truss_off[s] : 0, nt = in->truss_off ? in->truss_off[s + 1] - t0 : 0;
  if (!st && nt)
    st = fem_gpu_add_trusses(h, in->truss_numbers + t0, in->truss_nodes + 2 * t0, in->truss_young + t0,
                             in->truss_area + t0, in->truss_area2 ? in->truss_area2 + t0 : nullptr, nt, &n);
  const size_t b0 = in->beam_off ? in->beam_off[s] : 0, nb = in->beam_off ? in->beam_off[s + 1] - b0 : 0;
  if (!st && nb)
    st = fem_gpu_add_beams(h, in->beam_numbers + b0, in->beam_nodes + 2 * b0, in->beam_young + b0,
                           in->beam_poisson + b0, in->beam_area + b0, in->beam_i11 + b0, in->beam_i22 + b0,
                           in->beam_i12 + b0, in->beam_it + b0, in->beam_shear_factor + b0,
                           in->beam_local_axis + 3 * b0, nb, &n);
  const size_t p0 = in->plate_off ? in->plate_off[s] : 0, np = in->plate_off ? in->plate_off[s + 1] - p0 : 0;
  if (!st && np)
    st = fem_gpu_add_plates(h, in->plate_numbers + p0, in->plate_nodes + 4 * p0, in->plate_young + p0,
                            in->plate_poisson + p0, in->plate_thickness + p0, in->plate_shear_factor + p0, np, &n);
  if (st) *msg = fem_gpu_last_error(h);
  fem_gpu_destroy(h);
  return st;
}

// A caller's host array to the device.  Where the GPU reads pageable host memory itself
// (cudaDevAttrPageableMemoryAccess: address translation over the host link, as on Grace systems), a
// kernel reads it at the link's rate; a pageable cudaMemcpyAsync goes through the driver's staging, which
// took anywhere from 1.6 to 72 ms for the same 120 MB of coordinates between one call and the next.
// Small, unaligned or unreadable-in-place arrays take cudaMemcpyAsync.  Asynchronous either way: the
// caller's array must stay valid until the stream has passed the copy.
__global__ void k_read_host(const uint4* __restrict__ src, uint4* __restrict__ dst, size_t n16) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n16; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}
constexpr size_t kDirectReadBytes = 1u << 20;
cudaError_t host_to_device(void* dst, const void* src, size_t bytes, cudaStream_t s, int sm_count) {
  static std::atomic<int> direct[64];  // per device: 0 = not asked yet, 1 = reads in place, 2 = copies
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  int mode = 2;
  if (dev >= 0 && dev < 64) {
    mode = direct[dev].load(std::memory_order_relaxed);
    if (!mode) {
      int v = 0;
      if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) v = 0;
      mode = v ? 1 : 2;
      direct[dev].store(mode, std::memory_order_relaxed);
    }
  }
  const bool use = mode == 1 && bytes >= kDirectReadBytes && ((uintptr_t)src % 16) == 0 &&
                   ((uintptr_t)dst % 16) == 0;
  if (!use) return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s);
  const size_t n16 = bytes / 16, tail = bytes - n16 * 16;
  k_read_host<<<(unsigned)std::max(1, sm_count * 4), 256, 0, s>>>(static_cast<const uint4*>(src),
                                                                  static_cast<uint4*>(dst), n16);
  e = cudaGetLastError();
  if (e != cudaSuccess || !tail) return e;
  return cudaMemcpyAsync(static_cast<char*>(dst) + n16 * 16, static_cast<const char*>(src) + n16 * 16, tail,
                         cudaMemcpyHostToDevice, s);
}

// the element kinds of the input, in call order
struct BaKind {
  int kind;
  int per_el;                   // nodes per element
  const size_t* off;            // n_structures + 1 (NULL: none of this kind)
  const uint32_t* numbers;
  const uint32_t* nodes;
};

bool ba_offsets_ok(const size_t* off, size_t S) {
  if (!off) return true;
  if (off[0] != 0) return false;
  for (size_t s = 0; s < S; ++s)
    if (off[s + 1] < off[s]) return false;
  return true;
}

}  // namespace

extern "C" int fem_gpu_batch_create_from_arrays(double rel_tol, double abs_tol, const fem_gpu_structures_t* in,
                                                fem_gpu_batch_t** out) {
  if (!out || !in) return FEM_GPU_ERR_ARGUMENT;
  *out = nullptr;
  fem_gpu_batch* b = new fem_gpu_batch();
  *out = b;
  const auto t_start = std::chrono::steady_clock::now();
  auto mark = [&](int k) {
    b->build_ms[k] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
  };
  const size_t S = in->n_structures;
  if (S == 0 || S >= (1ull << 31) || !in->nodes_number || !in->node_off || !ba_offsets_ok(in->node_off, S) ||
      !ba_offsets_ok(in->truss_off, S) || !ba_offsets_ok(in->beam_off, S) || !ba_offsets_ok(in->plate_off, S))
    return b->fail(FEM_GPU_ERR_ARGUMENT, "structures: need n_structures >= 1 and nondecreasing offsets from 0");
  const size_t NN = in->node_off[S];
  const size_t NT = in->truss_off ? in->truss_off[S] : 0, NB = in->beam_off ? in->beam_off[S] : 0,
               NP = in->plate_off ? in->plate_off[S] : 0;
  if ((NN && (!in->node_numbers || !in->xyz)) ||
      (NT && (!in->truss_numbers || !in->truss_nodes || !in->truss_young || !in->truss_area)) ||
      (NB && (!in->beam_numbers || !in->beam_nodes || !in->beam_young || !in->beam_poisson || !in->beam_area ||
              !in->beam_i11 || !in->beam_i22 || !in->beam_i12 || !in->beam_it || !in->beam_shear_factor ||
              !in->beam_local_axis)) ||
      (NP && (!in->plate_numbers || !in->plate_nodes || !in->plate_young || !in->plate_poisson ||
              !in->plate_thickness || !in->plate_shear_factor)))
    return b->fail(FEM_GPU_ERR_ARGUMENT, "structures: a non-empty array is NULL");
  // node slots
  std::vector<unsigned long long> cap_off(S + 1, 0), node_off(S + 1);
  std::vector<int> fail(S, 0);
  for (size_t s = 0; s < S; ++s) {
    cap_off[s + 1] = cap_off[s] + in->nodes_number[s];
    node_off[s] = in->node_off[s];
    if (in->node_off[s + 1] - in->node_off[s] > in->nodes_number[s]) fail[s] = 1;  // more nodes than room
  }
  node_off[S] = in->node_off[S];
  const unsigned long long NS = cap_off[S];
  if (NS >= (1ull << 31) || NN >= (1ull << 32) || NT >= (1ull << 31) || NB >= (1ull << 31) || NP >= (1ull << 31))
    return b->fail(FEM_GPU_ERR_ARGUMENT, "structures: more than 2^31 node slots or elements of a kind in one batch");
  b->rel_tol = rel_tol;
  b->abs_tol = abs_tol;
  int dev = 0;
  BCK(cudaGetDevice(&dev));
  BCK(cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, dev));
  BCK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  for (auto& e : b->ev) BCK(cudaEventCreate(&e));
  BCK(b->flag.reserve(1, b->stream));
  BCK(b->counter.reserve(1, b->stream));
  // the union model: its handle, stream and node slots
  fem_gpu_t* U = nullptr;
  int st = fem_gpu_create(rel_tol, abs_tol, (uint32_t)NS, &U);
  if (st) return b->fail(st, "structures: creating the union model failed");
  b->un = U;
  fem_gpu* h = U;  // the CK macro reports through the union's handle
  st = ensure_ready(h);
  if (st) return b->fail(st, "%s", h->err.c_str());
  cudaStream_t s = h->stream;
  // Kernels on s read the caller's arrays in place (host_to_device); every return from here on, a failure
  // included, waits for s, so that nothing still reads them once the call is back.
  struct DrainOnReturn {
    cudaStream_t s;
    ~DrainOnReturn() {
      cudaStreamCaptureStatus c = cudaStreamCaptureStatusNone;
      if (cudaStreamIsCapturing(s, &c) == cudaSuccess && c == cudaStreamCaptureStatusNone) cudaStreamSynchronize(s);
    }
  } drain_on_return{s};
  auto cerr = [&](int code) { return b->fail(code, "%s", h->err.c_str()); };
#define BAK(call)                                     \
  do {                                                \
    cudaError_t e_ = (call);                          \
    if (e_ != cudaSuccess) return cerr(h->cuda_fail(e_, #call)); \
  } while (0)
  DevBuf<unsigned long long> d_capoff, d_nodeoff, d_eloff;
  DevBuf<int> d_fail;
  BAK(d_capoff.reserve(S + 1, s));
  BAK(d_nodeoff.reserve(S + 1, s));
  BAK(d_eloff.reserve(S + 1, s));
  BAK(d_fail.reserve(S, s));
  BAK(cudaMemcpyAsync(d_capoff.p, cap_off.data(), (S + 1) * sizeof(unsigned long long), cudaMemcpyHostToDevice, s));
  BAK(cudaMemcpyAsync(d_nodeoff.p, node_off.data(), (S + 1) * sizeof(unsigned long long), cudaMemcpyHostToDevice, s));
  BAK(cudaMemcpyAsync(d_fail.p, fail.data(), S * sizeof(int), cudaMemcpyHostToDevice, s));
  // sorts: keys + items, sorted copies
  DevBuf<unsigned long long> key, skey;
  DevBuf<uint32_t> idx, sidx, nsid, esid, u32;
  const size_t most = std::max<size_t>({NN, 4 * NP, 2 * NB, 2 * NT, 1});
  BAK(key.reserve(most, s));
  BAK(skey.reserve(most, s));
  BAK(idx.reserve(most, s));
  BAK(sidx.reserve(most, s));
  auto sort_pairs = [&](size_t n, int bits) -> int {
    return cub_call(h, [&](void* tmp, size_t& bytes) {
      return cub::DeviceRadixSort::SortPairs(tmp, bytes, key.p, skey.p, idx.p, sidx.p, (int64_t)n, 0, bits, s);
    });
  };
  int sbits = 1;
  while (sbits < 31 && (S >> sbits) != 0) ++sbits;
  // nodes: numbers repeated inside a structure, coordinates repeated inside a structure, slots
  BAK(nsid.reserve(NN + 1, s));
  BAK(u32.reserve(most + 1, s));
  BAK(h->stage.reserve(3 * NN + 1, s));
  if (NN) {
    BAK(host_to_device(u32.p, in->node_numbers, NN * sizeof(uint32_t), s, b->sm_count));
    BAK(host_to_device(h->stage.p, in->xyz, 3 * NN * sizeof(double), s, b->sm_count));
    k_ba_sid<<<grid_for(NN, 256), 256, 0, s>>>(d_nodeoff.p, (uint32_t)S, NN, nsid.p);
    k_ba_coord_keys<<<grid_for(NN, 256), 256, 0, s>>>(NN, nsid.p, h->stage.p, key.p, idx.p);
    st = sort_pairs(NN, 64);
    if (st) return cerr(st);
    k_ba_coord_dups<<<grid_for(NN, 256), 256, 0, s>>>(NN, skey.p, sidx.p, nsid.p, h->stage.p, d_fail.p);
  }
  BAK(h->dx.reserve(NS + 1, s));
  BAK(h->dy.reserve(NS + 1, s));
  BAK(h->dz.reserve(NS + 1, s));
  BAK(cudaMemsetAsync(h->dx.p, 0, (NS + 1) * sizeof(double), s));
  BAK(cudaMemsetAsync(h->dy.p, 0, (NS + 1) * sizeof(double), s));
  BAK(cudaMemsetAsync(h->dz.p, 0, (NS + 1) * sizeof(double), s));
  DevBuf<unsigned long long> nkey;
  DevBuf<uint32_t> nidx;
  BAK(nkey.reserve(NN + 1, s));
  BAK(nidx.reserve(NN + 1, s));
  if (NN) {
    k_ba_place_nodes<<<grid_for(NN, 256), 256, 0, s>>>(NN, nsid.p, h->stage.p, d_nodeoff.p, d_capoff.p, h->dx.p, h->dy.p,
                                                        h->dz.p);
    k_ba_num_keys<<<grid_for(NN, 256), 256, 0, s>>>(NN, nsid.p, u32.p, key.p, idx.p);
    st = sort_pairs(NN, 32 + sbits);
    if (st) return cerr(st);
    k_ba_equal_keys<<<grid_for(NN, 256), 256, 0, s>>>(NN, skey.p, sidx.p, nsid.p, d_fail.p);
    BAK(cudaMemcpyAsync(nkey.p, skey.p, NN * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, s));
    BAK(cudaMemcpyAsync(nidx.p, sidx.p, NN * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
  }
  BAK(cudaGetLastError());
  BAK(cudaStreamSynchronize(s));
  mark(0);
  // elements, kind by kind: numbers, nodes, properties, repeated numbers and node pairs / sets, validation
  const BaKind kinds[3] = {{kTruss, 2, in->truss_off, in->truss_numbers, in->truss_nodes},
                           {kBeam, 2, in->beam_off, in->beam_numbers, in->beam_nodes},
                           {kPlate, 4, in->plate_off, in->plate_numbers, in->plate_nodes}};
  DevBuf<double> v3;
  DevBuf<int> status;
  DevBuf<unsigned long long> first;
  BAK(first.reserve(1, s));
  for (const BaKind& k : kinds) {
    const size_t n = k.off ? k.off[S] : 0;
    if (!n) continue;
    std::vector<unsigned long long> eoff(S + 1);
    for (size_t q = 0; q <= S; ++q) eoff[q] = k.off[q];
    BAK(cudaMemcpyAsync(d_eloff.p, eoff.data(), (S + 1) * sizeof(unsigned long long), cudaMemcpyHostToDevice, s));
    BAK(esid.reserve(n + 1, s));
    k_ba_sid<<<grid_for(n, 256), 256, 0, s>>>(d_eloff.p, (uint32_t)S, n, esid.p);
    // element numbers repeated inside a structure
    BAK(host_to_device(u32.p, k.numbers, n * sizeof(uint32_t), s, b->sm_count));
    k_ba_num_keys<<<grid_for(n, 256), 256, 0, s>>>(n, esid.p, u32.p, key.p, idx.p);
    st = sort_pairs(n, 32 + sbits);
    if (st) return cerr(st);
    k_ba_equal_keys<<<grid_for(n, 256), 256, 0, s>>>(n, skey.p, sidx.p, esid.p, d_fail.p);
    // node numbers -> node slots
    BAK(host_to_device(u32.p, k.nodes, (size_t)k.per_el * n * sizeof(uint32_t), s, b->sm_count));
    int32_t* o[4] = {nullptr, nullptr, nullptr, nullptr};
    if (k.kind == kTruss) {
      BAK(h->t_n1.reserve(n + 1, s));
      BAK(h->t_n2.reserve(n + 1, s));
      o[0] = h->t_n1.p;
      o[1] = h->t_n2.p;
    } else if (k.kind == kBeam) {
      BAK(h->b_n1.reserve(n + 1, s));
      BAK(h->b_n2.reserve(n + 1, s));
      o[0] = h->b_n1.p;
      o[1] = h->b_n2.p;
    } else {
      for (DevBuf<int32_t>* d : {&h->p_n1, &h->p_n2, &h->p_n3, &h->p_n4}) BAK(d->reserve(n + 1, s));
      o[0] = h->p_n1.p;
      o[1] = h->p_n2.p;
      o[2] = h->p_n3.p;
      o[3] = h->p_n4.p;
    }
    if (!NN) {  // elements but no node anywhere: the first structure with elements fails
      for (size_t q = 0; q < S; ++q) {
        if (k.off[q + 1] == k.off[q]) continue;
        std::string msg;
        const int code = ba_replay(rel_tol, abs_tol, in, q, &msg);
        if (code) return b->fail(code, "structure %zu: %s", q, msg.c_str());
      }
    }
    k_ba_lookup<<<grid_for((size_t)k.per_el * n, 256), 256, 0, s>>>(n, k.per_el, esid.p, u32.p, nkey.p, nidx.p, NN,
                                                                    d_nodeoff.p, d_capoff.p, o[0], o[1], o[2], o[3],
                                                                    d_fail.p);
    // properties
    auto up = [&](DevBuf<double>& d, const double* src) -> int {
      BAK(d.reserve(n + 1, s));
      BAK(host_to_device(d.p, src, n * sizeof(double), s, b->sm_count));
      return FEM_GPU_OK;
    };
    int r = 0;
    if (k.kind == kTruss) {
      if ((r = up(h->t_E, in->truss_young)) || (r = up(h->t_A, in->truss_area))) return r;
      if (in->truss_area2) {
        if ((r = up(h->t_A2, in->truss_area2))) return r;
      } else {
        BAK(h->t_A2.reserve(n + 1, s));
        k_ba_fill<<<grid_for(n, 256), 256, 0, s>>>(n, __builtin_nan(""), h->t_A2.p);
      }
    } else if (k.kind == kBeam) {
      if ((r = up(h->b_E, in->beam_young)) || (r = up(h->b_nu, in->beam_poisson)) || (r = up(h->b_A, in->beam_area)) ||
          (r = up(h->b_i11, in->beam_i11)) || (r = up(h->b_i22, in->beam_i22)) || (r = up(h->b_i12, in->beam_i12)) ||
          (r = up(h->b_it, in->beam_it)) || (r = up(h->b_ks, in->beam_shear_factor)))
        return r;
      BAK(v3.reserve(3 * n + 1, s));
      BAK(host_to_device(v3.p, in->beam_local_axis, 3 * n * sizeof(double), s, b->sm_count));
      for (DevBuf<double>* d : {&h->b_ax, &h->b_ay, &h->b_az}) BAK(d->reserve(n + 1, s));
      k_ba_split3<<<grid_for(n, 256), 256, 0, s>>>(n, v3.p, h->b_ax.p, h->b_ay.p, h->b_az.p);
    } else {
      if ((r = up(h->p_E, in->plate_young)) || (r = up(h->p_nu, in->plate_poisson)) ||
          (r = up(h->p_t, in->plate_thickness)) || (r = up(h->p_ks, in->plate_shear_factor)))
        return r;
    }
    // repeated node pairs (two-node kinds) or node sets (plates)
    if (k.kind == kPlate) {
      k_set4_keys<<<grid_for(n, 256), 256, 0, s>>>(n, h->p_n1.p, h->p_n2.p, h->p_n3.p, h->p_n4.p, key.p, idx.p);
      st = sort_pairs(n, 64);
      if (st) return cerr(st);
      k_ba_set4_dups<<<grid_for(n, 256), 256, 0, s>>>(n, skey.p, sidx.p, h->p_n1.p, h->p_n2.p, h->p_n3.p, h->p_n4.p,
                                                       esid.p, d_fail.p);
    } else {
      k_ba_pair_keys<<<grid_for(n, 256), 256, 0, s>>>(n, o[0], o[1], key.p, idx.p);
      st = sort_pairs(n, 64);
      if (st) return cerr(st);
      k_ba_equal_keys<<<grid_for(n, 256), 256, 0, s>>>(n, skey.p, sidx.p, esid.p, d_fail.p);
    }
    // the plain path's validation of every element
    BAK(status.reserve(n + 1, s));
    const NodesView nd = h->nodes();
    if (k.kind == kTruss)
      k_validate_truss<<<grid_for(n, 128), 128, 0, s>>>(nd, h->t_n1.p, h->t_n2.p, h->t_E.p, h->t_A.p, h->t_A2.p, 0, n,
                                                        status.p, first.p);
    else if (k.kind == kBeam)
      k_validate_beam<<<grid_for(n, 128), 128, 0, s>>>(nd, h->beams(), 0, n, status.p, first.p);
    else
      k_validate_plate<<<grid_for(n, 128), 128, 0, s>>>(nd, h->plates(), abs_tol, 0, n, status.p, first.p);
    k_ba_status<<<grid_for(n, 256), 256, 0, s>>>(n, status.p, esid.p, d_fail.p);
    BAK(cudaGetLastError());
    BAK(cudaStreamSynchronize(s));  // the host offsets above are on this frame
    mark(1 + k.kind);
  }
  BAK(cudaMemcpyAsync(fail.data(), d_fail.p, S * sizeof(int), cudaMemcpyDeviceToHost, s));
  BAK(cudaStreamSynchronize(s));
  mark(4);
  for (size_t q = 0; q < S; ++q) {
    if (!fail[q]) continue;
    std::string msg;
    const int code = ba_replay(rel_tol, abs_tol, in, q, &msg);
    if (code) return b->fail(code, "structure %zu: %s", q, msg.c_str());
  }
  // the union model: every structure's elements in one run per kind (each structure's trusses come before
  // its beams, its beams before its plates), then its pattern and first values
  h->n_nodes = NS;
  h->nt = NT;
  h->nbm = NB;
  h->np = NP;
  h->append_run(kTruss, 0, NT);
  h->append_run(kBeam, 0, NB);
  h->append_run(kPlate, 0, NP);
  st = fem_gpu_assemble(h);
  if (st) return b->fail(st, "%s", h->err.c_str());
  mark(5);
  // per structure: entry offsets, local columns and row starts
  std::vector<int64_t> zoff(S + 1);
  DevBuf<int64_t> d_zoff;
  BAK(d_zoff.reserve(S + 1, s));
  k_ba_entry_offsets<<<grid_for(S + 1, 256), 256, 0, s>>>(S + 1, d_capoff.p, h->row_ptr.p, d_zoff.p);
  BAK(cudaMemcpyAsync(zoff.data(), d_zoff.p, (S + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  BAK(b->row_local.reserve(6 * NS + 1, s));
  if (NS)
    k_ba_localise<<<grid_for(6 * NS, 256), 256, 0, s>>>(6 * NS, d_capoff.p, (uint32_t)S, h->row_ptr.p, h->col_idx.p,
                                                        b->row_local.p);
  BAK(cudaGetLastError());
  BAK(cudaStreamSynchronize(s));
  for (size_t q = 0; q < S; ++q) {
    b->cap_off.push_back((size_t)cap_off[q]);
    b->cap_n.push_back((size_t)(cap_off[q + 1] - cap_off[q]));
    b->nnz_off.push_back(zoff[q]);
    b->nnz_n.push_back(zoff[q + 1] - zoff[q]);
  }
#undef BAK
  // the batch's numeric pass reads the union model's arrays
  b->n_nodes = NS;
  b->nt = NT;
  b->nbm = NB;
  b->np = NP;
  b->nnz = h->nnz;
  BatchData& d = b->d;
  d.nd = h->nodes();
  d.tv = h->trusses();
  d.bv = h->beams();
  d.pv = h->plates();
  d.pk_t = h->off_t.p;
  d.pk_b = h->off_b.p;
  d.pk_p = h->off_p.p;
  d.V = h->V.p;
  d.desc = h->slot_desc.p;
  d.n_desc = h->n_desc;
  d.n_sums = h->s_words;
  d.vs_off = h->vs_off;
  d.v_words = h->v_words;
  d.src_map = h->src_map.p;
  d.values = h->values.p;
  mark(6);
  st = batch_make_graph(b);
  mark(7);
  return st;
}

extern "C" int fem_gpu_batch_build_ms(const fem_gpu_batch_t* b, double* ms, size_t n) {
  if (!b || (n && !ms)) return FEM_GPU_ERR_ARGUMENT;
  for (size_t k = 0; k < n && k < 8; ++k) ms[k] = b->build_ms[k];
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_batch_size(const fem_gpu_batch_t* b, size_t* n_structures) {
  if (!b || !n_structures) return FEM_GPU_ERR_ARGUMENT;
  *n_structures = b->nnz_n.size();
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_batch_get_csr_sizes(fem_gpu_batch_t* b, size_t i, int64_t* n_rows, int64_t* nnz) {
  if (!b || i >= b->nnz_n.size()) return FEM_GPU_ERR_ARGUMENT;
  if (n_rows) *n_rows = b->un ? (int64_t)(6 * b->cap_n[i]) : (int64_t)6 * b->models[i]->nodes_number;
  if (nnz) *nnz = b->nnz_n[i];
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_batch_get_csr(fem_gpu_batch_t* b, size_t i, int64_t* row_ptr, int32_t* col_idx,
                                     double* values) {
  if (!b || i >= b->nnz_n.size()) return FEM_GPU_ERR_ARGUMENT;
  if (!b->un) {  // a union of models: the model's pattern, the batch's values
    fem_gpu* m = b->models[i];
    int st = fem_gpu_get_csr(m, row_ptr, col_idx, nullptr);
    if (st) return b->fail(st, "%s", m->err.c_str());
    return values ? fem_gpu_batch_get_values(b, i, values) : FEM_GPU_OK;
  }
  const size_t rows = 6 * b->cap_n[i];
  const int64_t z0 = b->nnz_off[i], nz = b->nnz_n[i];
  if (row_ptr) {
    if (rows)
      BCK(cudaMemcpyAsync(row_ptr, b->row_local.p + 6 * b->cap_off[i], rows * sizeof(int64_t), cudaMemcpyDeviceToHost,
                          b->stream));
  }
  if (col_idx && nz)
    BCK(cudaMemcpyAsync(col_idx, b->un->col_idx.p + z0, (size_t)nz * sizeof(int32_t), cudaMemcpyDeviceToHost,
                        b->stream));
  if (values && nz)
    BCK(cudaMemcpyAsync(values, b->d.values + z0, (size_t)nz * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  if (row_ptr) row_ptr[rows] = nz;
  return FEM_GPU_OK;
}
