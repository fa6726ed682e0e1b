// fem_batch.cuh -- batched assembly of many independent structures (included
// by fem_gpu.cu, whose kernels and handle it reuses).
//
// A batch is the disjoint union of assembled models: their nodes, elements,
// packed scratch, block-sum descriptors and CSR source maps are concatenated
// once (with node, scratch, slot and entry offsets applied on the device), so
// one numeric pass over the union assembles every structure -- the result for
// structure i is the slice [nnz_off[i], nnz_off[i] + nnz[i]) of the union's
// CSR values, with the model's own row_ptr / col_idx.  Each block's
// contributions come from one model and keep that model's element order, so
// every value is bit-identical to the model's own assembly.
//
// The numeric pass is captured once in a CUDA graph and replayed.  Its element
// phase is either one persistent launch (one CTA per SM slot pulls tiles of
// plates, beams and trusses from an atomic counter, one tile shape per element
// kind) or three plain launches, whichever the autotuner measures faster on the
// batch; the choice and the measured candidates are written to a JSON table
// keyed by the element mix and the SM count.

struct ElemTile {
  uint32_t kind;   // kTruss, kBeam, kPlate
  uint32_t count;  // elements in the tile
  unsigned long long start;
};

// Persistent element kernel: CTAs take tiles in list order until none is left.
// No waiting on other CTAs: a CTA that finds the list exhausted exits.
__global__ void __launch_bounds__(128) k_elements_persistent(NodesView nd, TrussView tv, BeamView bv, PlateView pv,
                                                             double rel_tol, double abs_tol, BlockSink st,
                                                             BlockSink sb, BlockSink sp,
                                                             const ElemTile* __restrict__ tiles, uint32_t n_tiles,
                                                             unsigned int* counter) {
  __shared__ uint32_t s_tile;
  for (;;) {
    if (threadIdx.x == 0) s_tile = atomicAdd(counter, 1u);
    __syncthreads();
    const uint32_t t = s_tile;
    __syncthreads();
    if (t >= n_tiles) return;
    const ElemTile tile = tiles[t];
    for (uint32_t i = threadIdx.x; i < tile.count; i += blockDim.x) {
      const size_t e = tile.start + i;
      if (tile.kind == kPlate) plate_element(e, nd, pv, abs_tol, sp);
      else if (tile.kind == kBeam) beam_element(e, nd, bv, rel_tol, abs_tol, sb);
      else truss_element(e, nd, tv, abs_tol, st);
    }
  }
}

// union fix-ups: shift node indices / scratch offsets / slot sources by per-model offsets
__global__ void k_add_i32(int32_t* a, size_t n, int32_t d) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) a[i] += d;
}
__global__ void k_add_pack(unsigned long long* a, size_t n, unsigned long long d) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) {
    const unsigned long long top = a[i] & (3ull << 62);
    a[i] = top | ((a[i] & ~(3ull << 62)) + d);
  }
}
__global__ void k_add_desc(uint2* a, size_t n, uint32_t d) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) a[i].x += d;
}
// model source s: below vs_off_m it is scratch (shift by the model's scratch
// offset), above it is an S slot (re-based into the union's S)
__global__ void k_fix_src(uint32_t* a, size_t n, uint32_t vs_off_m, uint32_t v_shift, uint32_t s_base) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < n) a[i] = a[i] < vs_off_m ? a[i] + v_shift : s_base + (a[i] - vs_off_m);
}

struct BatchConfig {
  int persistent = 0;      // 1: one persistent element launch
  int block = 128;         // threads per CTA of the plain element launches
  int ctas_per_sm = 2;     // persistent grid = SMs x this
  int tile[3] = {512, 256, 128};  // persistent tile size per kind (truss, beam, plate)
  int sum_block = 256;     // threads per CTA of the block sums / gather
};

// The device arrays one numeric pass of a batch reads and writes: owned by the
// batch (a union of assembled models) or by its union model (a batch built from
// host arrays).
struct BatchData {
  NodesView nd{};
  TrussView tv{};
  BeamView bv{};
  PlateView pv{};
  const unsigned long long *pk_t = nullptr, *pk_b = nullptr, *pk_p = nullptr;
  double* V = nullptr;
  const uint2* desc = nullptr;      // block-sum descriptors (sums first, then the check-only ones)
  size_t n_desc = 0, n_sums = 0;
  unsigned long long vs_off = 0;    // S starts here in V
  unsigned long long v_words = 0;   // packed element scratch (before S)
  const uint32_t* src_map = nullptr;
  double* values = nullptr;
};

struct fem_gpu_batch {
  std::vector<fem_gpu*> models;
  // a batch built from host arrays: the union model that holds every structure, each structure's node
  // slots [cap_off[i], cap_off[i] + cap_n[i]) and its row starts relative to its first entry
  fem_gpu* un = nullptr;
  std::vector<size_t> cap_off, cap_n;
  DevBuf<int64_t> row_local;
  double build_ms[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // fem_gpu_batch_create_from_arrays phase ends, ms from its start
  BatchData d;
  cudaStream_t stream = nullptr;
  std::string err;
  int sm_count = 0;
  double rel_tol = 0, abs_tol = 0;
  // union data
  size_t n_nodes = 0, nt = 0, nbm = 0, np = 0;
  DevBuf<double> dx, dy, dz;
  DevBuf<int32_t> t_n1, t_n2, b_n1, b_n2, p_n1, p_n2, p_n3, p_n4;
  DevBuf<double> t_E, t_A, t_A2, b_E, b_nu, b_A, b_i11, b_i22, b_i12, b_it, b_ks, b_ax, b_ay, b_az, p_E, p_nu, p_t,
      p_ks;
  DevBuf<unsigned long long> pk_t, pk_b, pk_p;
  DevBuf<uint2> desc;
  size_t n_desc = 0, n_sums = 0;
  DevBuf<double> V;
  unsigned long long vs_off = 0;
  DevBuf<uint32_t> src_map;
  DevBuf<double> values;
  int64_t nnz = 0;
  std::vector<int64_t> nnz_off, nnz_n;
  DevBuf<int> flag;
  DevBuf<ElemTile> tiles;
  uint32_t n_tiles = 0;
  DevBuf<unsigned int> counter;
  BatchConfig cfg;
  cudaGraphExec_t graph = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  float last_ms = 0;

  int fail(int code, const char* fmt, ...) {
    char b[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(b, sizeof b, fmt, ap);
    va_end(ap);
    err = b;
    return code;
  }
  int cuda_fail(cudaError_t e, const char* what) {
    cudaGetLastError();
    return fail(e == cudaErrorMemoryAllocation ? FEM_GPU_ERR_OUT_OF_MEMORY : FEM_GPU_ERR_CUDA, "CUDA error in %s: %s",
                what, cudaGetErrorString(e));
  }
  NodesView nodes() const { return NodesView{dx.p, dy.p, dz.p, n_nodes}; }
  TrussView trusses() const { return TrussView{t_n1.p, t_n2.p, t_E.p, t_A.p, t_A2.p}; }
  BeamView beams() const {
    return BeamView{b_n1.p, b_n2.p, b_E.p, b_nu.p, b_A.p, b_i11.p, b_i22.p, b_i12.p, b_it.p, b_ks.p, b_ax.p, b_ay.p, b_az.p};
  }
  PlateView plates() const { return PlateView{p_n1.p, p_n2.p, p_n3.p, p_n4.p, p_E.p, p_nu.p, p_t.p, p_ks.p}; }
};

#define BCK(call)                                        \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return b->cuda_fail(e_, #call); \
  } while (0)

namespace {

template <class T>
cudaError_t append_d2d(DevBuf<T>& dst, size_t at, const DevBuf<T>& src, size_t n, cudaStream_t s) {
  if (!n) return cudaSuccess;
  return cudaMemcpyAsync(dst.p + at, src.p, n * sizeof(T), cudaMemcpyDeviceToDevice, s);
}

int batch_build_tiles(fem_gpu_batch* b) {
  std::vector<ElemTile> tl;
  // heaviest work first: plates, then beams, then trusses
  const size_t counts[3] = {b->nt, b->nbm, b->np};
  for (int kind : {kPlate, kBeam, kTruss}) {
    const size_t ts = (size_t)std::max(32, b->cfg.tile[kind]);
    for (size_t s0 = 0; s0 < counts[kind]; s0 += ts)
      tl.push_back(ElemTile{(uint32_t)kind, (uint32_t)std::min(ts, counts[kind] - s0), (unsigned long long)s0});
  }
  b->n_tiles = (uint32_t)tl.size();
  BCK(b->tiles.reserve(tl.size() + 1, b->stream));
  if (!tl.empty())
    BCK(cudaMemcpyAsync(b->tiles.p, tl.data(), tl.size() * sizeof(ElemTile), cudaMemcpyHostToDevice, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  return FEM_GPU_OK;
}

// enqueue one numeric pass of the union on b->stream (captured into the graph)
int batch_enqueue(fem_gpu_batch* b) {
  cudaStream_t s = b->stream;
  BCK(cudaMemsetAsync(b->flag.p, 0, sizeof(int), s));
  const BatchData& d = b->d;
  BlockSink st{nullptr, d.V, d.pk_t, b->flag.p, d.v_words};
  BlockSink sb{nullptr, d.V, d.pk_b, b->flag.p, d.v_words};
  BlockSink sp{nullptr, d.V, d.pk_p, b->flag.p, d.v_words};
  if (b->cfg.persistent) {
    BCK(cudaMemsetAsync(b->counter.p, 0, sizeof(unsigned int), s));
    const unsigned grid = (unsigned)std::max(1, b->sm_count * b->cfg.ctas_per_sm);
    k_elements_persistent<<<grid, 128, 0, s>>>(d.nd, d.tv, d.bv, d.pv, b->rel_tol, b->abs_tol, st, sb, sp, b->tiles.p,
                                               b->n_tiles, b->counter.p);
  } else {
    const unsigned bs = (unsigned)b->cfg.block;
    if (b->np) k_plate<<<grid_for(b->np, bs), bs, plate_smem(sp, bs), s>>>(d.nd, d.pv, b->abs_tol, b->np, sp);
    if (b->nbm) k_beam<<<grid_for(b->nbm, bs), bs, 0, s>>>(d.nd, d.bv, b->rel_tol, b->abs_tol, b->nbm, sb);
    if (b->nt) k_truss<<<grid_for(b->nt, bs), bs, 0, s>>>(d.nd, d.tv, b->abs_tol, b->nt, st);
  }
  const unsigned rb = (unsigned)b->cfg.sum_block;
  if (d.n_desc)
    k_block_sums<<<block_sums_grid(d.n_desc, rb), rb, 0, s>>>(d.n_desc, d.n_sums, d.desc, d.V, d.V + d.vs_off, b->flag.p,
                                                       d.v_words);
  if (b->nnz)
    k_gather_values<<<grid_for(((size_t)b->nnz + kGatherPerThread - 1) / kGatherPerThread, rb), rb, 0, s>>>(
        (size_t)b->nnz, d.src_map, d.V, d.vs_off, d.values, b->flag.p, d.vs_off + d.n_sums);
  BCK(cudaGetLastError());
  return FEM_GPU_OK;
}

int batch_make_graph(fem_gpu_batch* b) {
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  int st = batch_build_tiles(b);
  if (st) return st;
  cudaGraph_t g = nullptr;
  BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  st = batch_enqueue(b);
  cudaError_t e = cudaStreamEndCapture(b->stream, &g);
  if (st) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  if (e != cudaSuccess) return b->cuda_fail(e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&b->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return b->cuda_fail(e, "cudaGraphInstantiate");
  return FEM_GPU_OK;
}

// time `reps` graph launches of the current configuration (ms per launch, median)
int batch_time(fem_gpu_batch* b, int reps, float* ms) {
  std::vector<float> t;
  for (int r = 0; r < reps + 2; ++r) {
    BCK(cudaEventRecord(b->ev[0], b->stream));
    BCK(cudaGraphLaunch(b->graph, b->stream));
    BCK(cudaEventRecord(b->ev[1], b->stream));
    BCK(cudaEventSynchronize(b->ev[1]));
    float x = 0;
    BCK(cudaEventElapsedTime(&x, b->ev[0], b->ev[1]));
    if (r >= 2) t.push_back(x);
  }
  std::sort(t.begin(), t.end());
  *ms = t[t.size() / 2];
  return FEM_GPU_OK;
}

std::string config_json(const BatchConfig& c) {
  char buf[256];
  snprintf(buf, sizeof buf,
           "{\"persistent\": %d, \"block\": %d, \"ctas_per_sm\": %d, \"tile_truss\": %d, \"tile_beam\": %d, "
           "\"tile_plate\": %d, \"sum_block\": %d}",
           c.persistent, c.block, c.ctas_per_sm, c.tile[kTruss], c.tile[kBeam], c.tile[kPlate], c.sum_block);
  return buf;
}

}  // namespace

extern "C" int fem_gpu_batch_create(fem_gpu_t* const* models, size_t n_models, fem_gpu_batch_t** out) {
  if (!out || (n_models && !models)) return FEM_GPU_ERR_ARGUMENT;
  *out = nullptr;
  fem_gpu_batch* b = new fem_gpu_batch();
  for (size_t i = 0; i < n_models; ++i) {
    fem_gpu* m = models[i];
    if (!m || !m->pattern_valid || !m->stream) {
      b->err = "every model must be assembled (fem_gpu_assemble) before it joins a batch";
      *out = b;
      return FEM_GPU_ERR_STATE;
    }
    b->models.push_back(m);
  }
  *out = b;
  int dev = 0;
  BCK(cudaGetDevice(&dev));
  BCK(cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, dev));
  BCK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  for (auto& e : b->ev) BCK(cudaEventCreate(&e));
  BCK(b->flag.reserve(1, b->stream));
  BCK(b->counter.reserve(1, b->stream));
  if (n_models) {
    b->rel_tol = b->models[0]->rel_tol;
    b->abs_tol = b->models[0]->abs_tol;
  }
  // sizes and offsets
  size_t nn = 0, nt = 0, nbm = 0, np = 0, nsum = 0, nchk = 0;
  unsigned long long vw = 0;
  int64_t nz = 0;
  for (fem_gpu* m : b->models) {
    if (m->rel_tol != b->rel_tol || m->abs_tol != b->abs_tol) {
      b->err = "all models of a batch must share rel_tol and abs_tol";
      return FEM_GPU_ERR_ARGUMENT;
    }
    nn += m->n_nodes;
    nt += m->nt;
    nbm += m->nbm;
    np += m->np;
    nsum += m->s_words;
    nchk += m->n_desc - m->s_words;
    vw += ((unsigned long long)m->v_words + 3ull) & ~3ull;
    b->nnz_off.push_back(nz);
    b->nnz_n.push_back(m->nnz);
    nz += m->nnz;
  }
  b->n_nodes = nn;
  b->nt = nt;
  b->nbm = nbm;
  b->np = np;
  b->n_sums = nsum;
  b->n_desc = nsum + nchk;
  b->vs_off = vw;
  b->nnz = nz;
  if (b->vs_off + b->n_sums + 4 >= (1ull << 32)) {
    b->err = "batch too large: more than 2^32 doubles of scratch and sums";
    return FEM_GPU_ERR_ARGUMENT;
  }
  cudaStream_t s = b->stream;
  BCK(b->dx.reserve(nn + 1, s));
  BCK(b->dy.reserve(nn + 1, s));
  BCK(b->dz.reserve(nn + 1, s));
  BCK(b->t_n1.reserve(nt + 1, s));
  BCK(b->t_n2.reserve(nt + 1, s));
  for (DevBuf<double>* d : {&b->t_E, &b->t_A, &b->t_A2}) BCK(d->reserve(nt + 1, s));
  BCK(b->b_n1.reserve(nbm + 1, s));
  BCK(b->b_n2.reserve(nbm + 1, s));
  for (DevBuf<double>* d : {&b->b_E, &b->b_nu, &b->b_A, &b->b_i11, &b->b_i22, &b->b_i12, &b->b_it, &b->b_ks, &b->b_ax,
                            &b->b_ay, &b->b_az})
    BCK(d->reserve(nbm + 1, s));
  for (DevBuf<int32_t>* d : {&b->p_n1, &b->p_n2, &b->p_n3, &b->p_n4}) BCK(d->reserve(np + 1, s));
  for (DevBuf<double>* d : {&b->p_E, &b->p_nu, &b->p_t, &b->p_ks}) BCK(d->reserve(np + 1, s));
  BCK(b->pk_t.reserve(nt * kPairs2 + 1, s));
  BCK(b->pk_b.reserve(nbm * kPairs2 + 1, s));
  BCK(b->pk_p.reserve(np * kPairs4 + 1, s));
  BCK(b->desc.reserve(b->n_desc + 1, s));
  BCK(b->V.reserve(b->vs_off + b->n_sums + 4, s));
  BCK(b->src_map.reserve((size_t)nz + 8, s));
  BCK(b->values.reserve((size_t)nz + 8, s));
  size_t on = 0, ot = 0, ob = 0, op = 0, osum = 0, ochk = nsum;
  unsigned long long ov = 0;
  int64_t oz = 0;
  for (fem_gpu* m : b->models) {
    BCK(append_d2d(b->dx, on, m->dx, m->n_nodes, s));
    BCK(append_d2d(b->dy, on, m->dy, m->n_nodes, s));
    BCK(append_d2d(b->dz, on, m->dz, m->n_nodes, s));
    // trusses
    BCK(append_d2d(b->t_n1, ot, m->t_n1, m->nt, s));
    BCK(append_d2d(b->t_n2, ot, m->t_n2, m->nt, s));
    BCK(append_d2d(b->t_E, ot, m->t_E, m->nt, s));
    BCK(append_d2d(b->t_A, ot, m->t_A, m->nt, s));
    BCK(append_d2d(b->t_A2, ot, m->t_A2, m->nt, s));
    BCK(append_d2d(b->pk_t, ot * kPairs2, m->off_t, m->nt * kPairs2, s));
    if (m->nt) {
      k_add_i32<<<grid_for(m->nt, 256), 256, 0, s>>>(b->t_n1.p + ot, m->nt, (int32_t)on);
      k_add_i32<<<grid_for(m->nt, 256), 256, 0, s>>>(b->t_n2.p + ot, m->nt, (int32_t)on);
      k_add_pack<<<grid_for(m->nt * kPairs2, 256), 256, 0, s>>>(b->pk_t.p + ot * kPairs2, m->nt * kPairs2, ov);
    }
    // beams
    BCK(append_d2d(b->b_n1, ob, m->b_n1, m->nbm, s));
    BCK(append_d2d(b->b_n2, ob, m->b_n2, m->nbm, s));
    DevBuf<double>* bd[] = {&b->b_E, &b->b_nu, &b->b_A, &b->b_i11, &b->b_i22, &b->b_i12, &b->b_it, &b->b_ks,
                            &b->b_ax, &b->b_ay, &b->b_az};
    DevBuf<double>* md[] = {&m->b_E, &m->b_nu, &m->b_A, &m->b_i11, &m->b_i22, &m->b_i12, &m->b_it, &m->b_ks,
                            &m->b_ax, &m->b_ay, &m->b_az};
    for (int k = 0; k < 11; ++k) BCK(append_d2d(*bd[k], ob, *md[k], m->nbm, s));
    BCK(append_d2d(b->pk_b, ob * kPairs2, m->off_b, m->nbm * kPairs2, s));
    if (m->nbm) {
      k_add_i32<<<grid_for(m->nbm, 256), 256, 0, s>>>(b->b_n1.p + ob, m->nbm, (int32_t)on);
      k_add_i32<<<grid_for(m->nbm, 256), 256, 0, s>>>(b->b_n2.p + ob, m->nbm, (int32_t)on);
      k_add_pack<<<grid_for(m->nbm * kPairs2, 256), 256, 0, s>>>(b->pk_b.p + ob * kPairs2, m->nbm * kPairs2, ov);
    }
    // plates
    DevBuf<int32_t>* pn[] = {&b->p_n1, &b->p_n2, &b->p_n3, &b->p_n4};
    DevBuf<int32_t>* mn[] = {&m->p_n1, &m->p_n2, &m->p_n3, &m->p_n4};
    for (int k = 0; k < 4; ++k) {
      BCK(append_d2d(*pn[k], op, *mn[k], m->np, s));
      if (m->np) k_add_i32<<<grid_for(m->np, 256), 256, 0, s>>>(pn[k]->p + op, m->np, (int32_t)on);
    }
    DevBuf<double>* pd[] = {&b->p_E, &b->p_nu, &b->p_t, &b->p_ks};
    DevBuf<double>* mp[] = {&m->p_E, &m->p_nu, &m->p_t, &m->p_ks};
    for (int k = 0; k < 4; ++k) BCK(append_d2d(*pd[k], op, *mp[k], m->np, s));
    BCK(append_d2d(b->pk_p, op * kPairs4, m->off_p, m->np * kPairs4, s));
    if (m->np)
      k_add_pack<<<grid_for(m->np * kPairs4, 256), 256, 0, s>>>(b->pk_p.p + op * kPairs4, m->np * kPairs4, ov);
    // block-sum descriptors: S slots first (all models), then the check-only ones
    if (m->s_words) {
      BCK(cudaMemcpyAsync(b->desc.p + osum, m->slot_desc.p, m->s_words * sizeof(uint2), cudaMemcpyDeviceToDevice, s));
      k_add_desc<<<grid_for(m->s_words, 256), 256, 0, s>>>(b->desc.p + osum, m->s_words, (uint32_t)ov);
    }
    const size_t nck = m->n_desc - m->s_words;
    if (nck) {
      BCK(cudaMemcpyAsync(b->desc.p + ochk, m->slot_desc.p + m->s_words, nck * sizeof(uint2),
                          cudaMemcpyDeviceToDevice, s));
      k_add_desc<<<grid_for(nck, 256), 256, 0, s>>>(b->desc.p + ochk, nck, (uint32_t)ov);
    }
    // CSR sources
    if (m->nnz) {
      BCK(cudaMemcpyAsync(b->src_map.p + oz, m->src_map.p, (size_t)m->nnz * sizeof(uint32_t),
                          cudaMemcpyDeviceToDevice, s));
      k_fix_src<<<grid_for((size_t)m->nnz, 256), 256, 0, s>>>(b->src_map.p + oz, (size_t)m->nnz, (uint32_t)m->vs_off,
                                                              (uint32_t)ov, (uint32_t)(b->vs_off + osum));
    }
    BCK(cudaGetLastError());
    on += m->n_nodes;
    ot += m->nt;
    ob += m->nbm;
    op += m->np;
    osum += m->s_words;
    ochk += nck;
    ov += ((unsigned long long)m->v_words + 3ull) & ~3ull;
    oz += m->nnz;
  }
  BCK(cudaStreamSynchronize(s));
  BatchData& d = b->d;
  d.nd = b->nodes();
  d.tv = b->trusses();
  d.bv = b->beams();
  d.pv = b->plates();
  d.pk_t = b->pk_t.p;
  d.pk_b = b->pk_b.p;
  d.pk_p = b->pk_p.p;
  d.V = b->V.p;
  d.desc = b->desc.p;
  d.n_desc = b->n_desc;
  d.n_sums = b->n_sums;
  d.vs_off = b->vs_off;
  d.v_words = b->vs_off;  // the models' scratch, end to end (S follows)
  d.src_map = b->src_map.p;
  d.values = b->values.p;
  BCK(cudaStreamSynchronize(s));
  return batch_make_graph(b);
}

extern "C" int fem_gpu_batch_destroy(fem_gpu_batch_t* b) {
  if (!b) return FEM_GPU_OK;
  cudaDeviceSynchronize();  // device pointers were handed out: all work must be done before the pool reuses them
  if (b->graph) cudaGraphExecDestroy(b->graph);
  DevBuf<double>* d[] = {&b->dx, &b->dy, &b->dz, &b->t_E, &b->t_A, &b->t_A2, &b->b_E, &b->b_nu, &b->b_A, &b->b_i11,
                         &b->b_i22, &b->b_i12, &b->b_it, &b->b_ks, &b->b_ax, &b->b_ay, &b->b_az, &b->p_E, &b->p_nu,
                         &b->p_t, &b->p_ks, &b->V, &b->values};
  for (auto* x : d) x->release();
  DevBuf<int32_t>* i[] = {&b->t_n1, &b->t_n2, &b->b_n1, &b->b_n2, &b->p_n1, &b->p_n2, &b->p_n3, &b->p_n4};
  for (auto* x : i) x->release();
  b->pk_t.release();
  b->pk_b.release();
  b->pk_p.release();
  b->desc.release();
  b->src_map.release();
  b->flag.release();
  b->tiles.release();
  b->counter.release();
  b->row_local.release();
  for (auto& e : b->ev)
    if (e) cudaEventDestroy(e);
  if (b->un) fem_gpu_destroy(b->un);
  cudaStream_t s = b->stream;
  delete b;  // the remaining device arrays are freed in the stream's order: the stream goes last
  if (s) cudaStreamDestroy(s);
  return FEM_GPU_OK;
}

extern "C" const char* fem_gpu_batch_last_error(const fem_gpu_batch_t* b) { return b ? b->err.c_str() : "null batch"; }

extern "C" int fem_gpu_batch_assemble_async(fem_gpu_batch_t* b) {
  if (!b || !b->graph) return FEM_GPU_ERR_ARGUMENT;
  BCK(cudaGraphLaunch(b->graph, b->stream));
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_batch_assemble(fem_gpu_batch_t* b) {
  if (!b || !b->graph) return FEM_GPU_ERR_ARGUMENT;
  BCK(cudaEventRecord(b->ev[0], b->stream));
  BCK(cudaGraphLaunch(b->graph, b->stream));
  BCK(cudaEventRecord(b->ev[1], b->stream));
  int flag = 0;
  BCK(cudaMemcpyAsync(&flag, b->flag.p, sizeof flag, cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  BCK(cudaEventElapsedTime(&b->last_ms, b->ev[0], b->ev[1]));
  if (flag)
    return b->fail(FEM_GPU_ERR_PATTERN_CHANGED,
                   "a structure's exact-zero pattern changed: reassemble it and build the batch again");
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_batch_get_values(fem_gpu_batch_t* b, size_t i, double* values) {
  if (!b || i >= b->nnz_n.size() || (!values && b->nnz_n[i])) return FEM_GPU_ERR_ARGUMENT;
  if (b->nnz_n[i])
    BCK(cudaMemcpyAsync(values, b->d.values + b->nnz_off[i], (size_t)b->nnz_n[i] * sizeof(double),
                        cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_batch_get_values_device(fem_gpu_batch_t* b, size_t i, const double** values) {
  if (!b || i >= b->nnz_n.size() || !values) return FEM_GPU_ERR_ARGUMENT;
  *values = b->d.values + b->nnz_off[i];
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_batch_get_stream(fem_gpu_batch_t* b, void** stream) {
  if (!b || !stream) return FEM_GPU_ERR_ARGUMENT;
  *stream = (void*)b->stream;
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_batch_last_ms(fem_gpu_batch_t* b, float* ms) {
  if (!b || !ms) return FEM_GPU_ERR_ARGUMENT;
  *ms = b->last_ms;
  return FEM_GPU_OK;
}

// Autotune: time each candidate configuration on this batch (CUDA graph
// replays, median of `reps`), keep the fastest, and write the table of
// candidates and the choice as JSON to `cache_path` (if given) and to
// `summary` (if given, truncated to `cap` bytes).
extern "C" int fem_gpu_batch_autotune(fem_gpu_batch_t* b, int reps, const char* cache_path, char* summary,
                                      size_t cap) {
  if (!b) return FEM_GPU_ERR_ARGUMENT;
  if (reps < 1) reps = 5;
  std::vector<BatchConfig> cand;
  for (int bs : {64, 128, 256}) {
    BatchConfig c;
    c.persistent = 0;
    c.block = bs;
    cand.push_back(c);
  }
  const int tiles[][3] = {{512, 256, 128}, {1024, 512, 256}, {2048, 1024, 512}, {4096, 2048, 1024}};
  for (int cps : {1, 2})
    for (const auto& t : tiles) {
      BatchConfig c;
      c.persistent = 1;
      c.ctas_per_sm = cps;
      c.tile[kTruss] = t[0];
      c.tile[kBeam] = t[1];
      c.tile[kPlate] = t[2];
      cand.push_back(c);
    }
  const BatchConfig keep = b->cfg;
  std::string rows;
  float best = 1e30f;
  BatchConfig best_cfg = keep;
  for (size_t k = 0; k < cand.size(); ++k) {
    BatchConfig c = cand[k];
    c.sum_block = keep.sum_block;
    b->cfg = c;
    int st = batch_make_graph(b);
    if (st) return st;
    float ms = 0;
    st = batch_time(b, reps, &ms);
    if (st) return st;
    char row[320];
    snprintf(row, sizeof row, "%s{\"config\": %s, \"ms\": %.4f}", k ? ", " : "", config_json(c).c_str(), ms);
    rows += row;
    if (ms < best) {
      best = ms;
      best_cfg = c;
    }
  }
  // the reduction's block size, with the best element phase
  for (int rb : {128, 512}) {
    BatchConfig c = best_cfg;
    c.sum_block = rb;
    b->cfg = c;
    int st = batch_make_graph(b);
    if (st) return st;
    float ms = 0;
    st = batch_time(b, reps, &ms);
    if (st) return st;
    char row[320];
    snprintf(row, sizeof row, ", {\"config\": %s, \"ms\": %.4f}", config_json(c).c_str(), ms);
    rows += row;
    if (ms < best) {
      best = ms;
      best_cfg = c;
    }
  }
  b->cfg = best_cfg;
  int st = batch_make_graph(b);
  if (st) return st;
  char head[512];
  snprintf(head, sizeof head,
           "{\"sm_count\": %d, \"structures\": %zu, \"elements\": {\"truss\": %zu, \"beam\": %zu, \"plate\": %zu}, "
           "\"best\": %s, \"best_ms\": %.4f, \"candidates\": [",
           b->sm_count, b->nnz_n.size(), b->nt, b->nbm, b->np, config_json(best_cfg).c_str(), best);
  std::string js = std::string(head) + rows + "]}";
  if (cache_path && *cache_path) {
    FILE* f = fopen(cache_path, "w");
    if (f) {
      fputs(js.c_str(), f);
      fputc('\n', f);
      fclose(f);
    }
  }
  if (summary && cap) {
    strncpy(summary, js.c_str(), cap - 1);
    summary[cap - 1] = 0;
  }
  return FEM_GPU_OK;
}

// Apply a configuration chosen earlier (for instance read back from the
// autotuner's JSON table): persistent 0/1, plain-launch block size, persistent
// CTAs per SM, tile sizes (truss, beam, plate) and the reduction block size.
extern "C" int fem_gpu_batch_configure(fem_gpu_batch_t* b, int persistent, int block, int ctas_per_sm, int tile_truss,
                                       int tile_beam, int tile_plate, int sum_block) {
  if (!b || (block != 64 && block != 128 && block != 256) || ctas_per_sm < 1 || ctas_per_sm > 8 ||
      (sum_block != 128 && sum_block != 256 && sum_block != 512) || tile_truss < 32 || tile_beam < 32 ||
      tile_plate < 32)
    return FEM_GPU_ERR_ARGUMENT;
  b->cfg.persistent = persistent ? 1 : 0;
  b->cfg.block = block;
  b->cfg.ctas_per_sm = ctas_per_sm;
  b->cfg.tile[kTruss] = tile_truss;
  b->cfg.tile[kBeam] = tile_beam;
  b->cfg.tile[kPlate] = tile_plate;
  b->cfg.sum_block = sum_block;
  return batch_make_graph(b);
}
