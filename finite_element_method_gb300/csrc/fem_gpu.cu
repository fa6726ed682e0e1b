// fem_gpu.cu -- GB300 (sm_103a) implementation of the C ABI in include/fem_gpu.h.
//
// Pipeline (one handle = one model = one CUDA stream):
//   add_*      host registries (node numbers, duplicates) as in the reference's
//              check_* functions, then a GPU validation kernel over the batch
//              (Truss/Beam/Plate::create checks); first failure wins.
//   symbolic   node-pair keys of every element in call order -> stable radix
//              sort -> global blocks (unordered node pairs) with their
//              contributors in element order; per-pair 36-bit non-zero masks
//              (from the numeric element arithmetic) -> block masks -> CSR
//              pattern, stiffness groups and the contribution map.
//   numeric    element kernels write each node-pair 6x6 block to its
//              destination-sorted slot (no atomics); the block reduction sums
//              the slots of a block in element order (bit-exact with the
//              reference's call-order accumulation) and scatters into CSR.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <condition_variable>
#include <cub/cub.cuh>
#include <functional>
#include <mutex>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <thread>
#include <vector>

#include <unistd.h>

#include "../../include/fem_gpu.h"
#include "element_math.cuh"

using namespace femgpu;

namespace {

constexpr int kTruss = 0, kBeam = 1, kPlate = 2;
constexpr int kPairs2 = 3;   // (1,1) (1,2) (2,2)
constexpr int kPairs4 = 10;  // (1,1) (1,2) (1,3) (1,4) (2,2) (2,3) (2,4) (3,3) (3,4) (4,4)

__host__ __device__ __forceinline__ void pair_nodes4(int p, int& i, int& j) {
  const int I[10] = {0, 0, 0, 0, 1, 1, 1, 2, 2, 3};
  const int J[10] = {0, 1, 2, 3, 1, 2, 3, 2, 3, 3};
  i = I[p];
  j = J[p];
}
__host__ __device__ __forceinline__ void pair_nodes2(int p, int& i, int& j) {
  i = p == 2 ? 1 : 0;
  j = p == 0 ? 0 : 1;
}

// ---------------------------------------------------------------------------
// device buffers
// ---------------------------------------------------------------------------
// Device memory comes from one stream-ordered pool per device that keeps what is freed (release threshold
// at its maximum): a model's buffers and an assembly's temporaries are served again without cudaMalloc /
// cudaFree, which cost milliseconds at these sizes and synchronise the device.
// fem_gpu_release_cached_memory hands the cached memory back.
std::mutex g_pool_mutex;
cudaMemPool_t g_pools[64] = {};

cudaError_t device_pool(cudaMemPool_t* out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_pool_mutex);
  if (!g_pools[dev]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool = nullptr;
    e = cudaMemPoolCreate(&pool, &props);
    if (e != cudaSuccess) return e;
    uint64_t keep_all = ~0ull;
    e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep_all);
    if (e != cudaSuccess) return e;
    g_pools[dev] = pool;
  }
  *out = g_pools[dev];
  return cudaSuccess;
}

// A device array owned by one object and used on one stream: allocated and freed in that stream's order.
template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t cap = 0;
  cudaStream_t st = nullptr;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  cudaError_t reserve(size_t n, cudaStream_t s, size_t keep = 0) {
    if (n <= cap) return cudaSuccess;
    size_t nc = std::max<size_t>(n, cap ? cap + cap / 2 : 256);
    cudaMemPool_t pool = nullptr;
    cudaError_t e = device_pool(&pool);
    if (e != cudaSuccess) return e;
    T* q = nullptr;
    e = cudaMallocFromPoolAsync((void**)&q, nc * sizeof(T), pool, s);
    if (e != cudaSuccess) return e;
    if (p) {
      if (st != s && st) {  // the old array's last uses were ordered on another stream
        e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return e;
      }
      if (keep) {
        e = cudaMemcpyAsync(q, p, keep * sizeof(T), cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) return e;
      }
      cudaFreeAsync(p, s);
    }
    p = q;
    cap = nc;
    st = s;
    return cudaSuccess;
  }
  void release() {
    if (p) cudaFreeAsync(p, st);
    p = nullptr;
    cap = 0;
  }
};

// ---------------------------------------------------------------------------
// kernels: validation
// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// debug builds: index checks on the assembly path
// ---------------------------------------------------------------------------
// Built with -DFEM_GPU_DEBUG (lib/libfem_gpu_debug.so), the assembly kernels
// check every node index, scratch position, block-sum source, CSR source and
// CSR / group position against the length of its array before the access.  An
// index out of range skips the access and records the first failing site,
// index and bound in g_dbg -- no trap, so the context stays usable and the host
// reads the record with fem_gpu_debug_check.  Without the macro the checks
// compile to nothing.
struct DebugRecord {
  int flag, site;
  unsigned long long index, bound;
};
__device__ DebugRecord g_dbg;
enum : int {
  kDbgNode = 1,         // node index of an element (coordinate gather)
  kDbgScratch = 2,      // packed block written by an element kernel
  kDbgSumSource = 3,    // last contribution read by a block sum
  kDbgGatherSource = 4, // scratch or sum slot read by the CSR gather
  kDbgCsrEntry = 5,     // CSR position written by the row fill
  kDbgGroup = 6,        // stiffness-group position written by the row fill
  kDbgRowSource = 7     // value source the row fill records for a CSR entry
};
constexpr unsigned long long kNoBound = ~0ull;
__device__ __forceinline__ bool dbg_in_range(unsigned long long i, unsigned long long n, int site) {
#ifdef FEM_GPU_DEBUG
  if (i < n) return true;
  if (atomicCAS(&g_dbg.flag, 0, 1) == 0) {
    g_dbg.site = site;
    g_dbg.index = i;
    g_dbg.bound = n;
  }
  return false;
#else
  (void)i;
  (void)n;
  (void)site;
  return true;
#endif
}

struct NodesView {
  const double *x, *y, *z;
  unsigned long long n = kNoBound;  // nodes held (checked in debug builds)
  __device__ __forceinline__ void get(int i, double o[3]) const {
    if (!dbg_in_range((unsigned long long)(unsigned)i, n, kDbgNode)) {
      o[0] = o[1] = o[2] = 0.0;
      return;
    }
    o[0] = x[i];
    o[1] = y[i];
    o[2] = z[i];
  }
};

// interleaved (x, y, z) rows -> the structure-of-arrays coordinates
__global__ void k_split_xyz(size_t n, const double* __restrict__ xyz, double* __restrict__ x, double* __restrict__ y,
                            double* __restrict__ z) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  x[i] = xyz[3 * i];
  y[i] = xyz[3 * i + 1];
  z[i] = xyz[3 * i + 2];
}

__global__ void k_validate_truss(NodesView nd, const int32_t* __restrict__ n1, const int32_t* __restrict__ n2,
                                 const double* __restrict__ E, const double* __restrict__ A,
                                 const double* __restrict__ A2, size_t begin, size_t count, int* status,
                                 unsigned long long* first) {
  size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k >= count) return;
  size_t e = begin + k;
  int st = 0;
  if (E[e] <= 0.0) st = FEM_GPU_ERR_YOUNG;
  else if (A[e] <= 0.0) st = FEM_GPU_ERR_AREA;
  else if (A2[e] == A2[e] && A2[e] <= 0.0) st = FEM_GPU_ERR_AREA2;
  else {
    double x1[3], x2[3], R[9];
    nd.get(n1[e], x1);
    nd.get(n2[e], x2);
    if (!truss_rotation(x1, x2, 0.0, R)) st = FEM_GPU_ERR_ZERO_LENGTH;
  }
  status[k] = st;
  if (st) atomicMin(first, (unsigned long long)k);
}

struct BeamView {
  const int32_t *n1, *n2;
  const double *E, *nu, *A, *i11, *i22, *i12, *it, *ks, *ax, *ay, *az;
};

__global__ void k_validate_beam(NodesView nd, BeamView b, size_t begin, size_t count, int* status,
                                unsigned long long* first) {
  size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k >= count) return;
  size_t e = begin + k;
  int st = 0;
  if (b.E[e] <= 0.0) st = FEM_GPU_ERR_YOUNG;
  else if (b.nu[e] <= 0.0) st = FEM_GPU_ERR_POISSON;
  else if (b.A[e] <= 0.0) st = FEM_GPU_ERR_AREA;
  else if (b.i11[e] <= 0.0) st = FEM_GPU_ERR_I11;
  else if (b.i22[e] <= 0.0) st = FEM_GPU_ERR_I22;
  else if (b.it[e] <= 0.0) st = FEM_GPU_ERR_IT;
  else if (b.ks[e] <= 0.0) st = FEM_GPU_ERR_SHEAR_FACTOR;
  else {
    double x1[3], x2[3], d[3], p[3];
    nd.get(b.n1[e], x1);
    nd.get(b.n2[e], x2);
    sub3(x2, x1, d);
    double axis[3] = {b.ax[e], b.ay[e], b.az[e]};
    project_perp(axis, d, p);
    if (norm3(p) == 0.0) st = FEM_GPU_ERR_PARALLEL_AXIS;
    else if (!(norm3(d) > 0.0)) st = FEM_GPU_ERR_ZERO_LENGTH;
  }
  status[k] = st;
  if (st) atomicMin(first, (unsigned long long)k);
}

struct PlateView {
  const int32_t *n1, *n2, *n3, *n4;
  const double *E, *nu, *t, *ks;
};

__global__ void k_validate_plate(NodesView nd, PlateView pl, double abs_tol, size_t begin, size_t count, int* status,
                                 unsigned long long* first) {
  size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k >= count) return;
  size_t e = begin + k;
  int st = 0;
  if (pl.E[e] <= 0.0) st = FEM_GPU_ERR_YOUNG;
  else if (pl.nu[e] <= 0.0) st = FEM_GPU_ERR_POISSON;
  else if (pl.t[e] <= 0.0) st = FEM_GPU_ERR_THICKNESS;
  else if (pl.ks[e] <= 0.0) st = FEM_GPU_ERR_SHEAR_FACTOR;
  else {
    double p1[3], p2[3], p3[3], p4[3];
    nd.get(pl.n1[e], p1);
    nd.get(pl.n2[e], p2);
    nd.get(pl.n3[e], p3);
    nd.get(pl.n4[e], p4);
    if (quad_on_line(p1, p2, p3, p4)) st = FEM_GPU_ERR_NODES_ON_LINE;
    else if (!quad_on_plane(p1, p2, p3, p4, abs_tol)) st = FEM_GPU_ERR_NOT_ON_PLANE;
    else {
      bool ok;
      int hs = quad_hull_size(p1, p2, p3, p4, abs_tol, ok);
      if (!ok) st = FEM_GPU_ERR_NODES_ON_LINE;
      else if (hs != 4) st = FEM_GPU_ERR_NOT_CONVEX;
    }
  }
  status[k] = st;
  if (st) atomicMin(first, (unsigned long long)k);
}

// rotation getters (fem.rs:171-202)
__global__ void k_rotation(int kind, NodesView nd, const int32_t* n1, const int32_t* n2, const int32_t* n3,
                           const int32_t* n4, BeamView b, double rel_tol, double abs_tol, size_t e, double* out) {
  double R[9];
  for (int k = 0; k < 9; ++k) R[k] = 0.0;
  if (kind == kTruss) {
    double x1[3], x2[3];
    nd.get(n1[e], x1);
    nd.get(n2[e], x2);
    truss_rotation(x1, x2, abs_tol, R);
  } else if (kind == kBeam) {
    double x1[3], x2[3], i11p, i22p;
    nd.get(b.n1[e], x1);
    nd.get(b.n2[e], x2);
    double axis[3] = {b.ax[e], b.ay[e], b.az[e]};
    beam_rotation(x1, x2, b.i11[e], b.i22[e], b.i12[e], axis, rel_tol, abs_tol, R, i11p, i22p);
  } else {
    double x2[3], x3[3], x4[3];
    nd.get(n2[e], x2);
    nd.get(n3[e], x3);
    nd.get(n4[e], x4);
    plate_rotation(x2, x3, x4, abs_tol, R);
  }
  for (int k = 0; k < 9; ++k) out[k] = R[k];
}

// ---------------------------------------------------------------------------
// kernels: symbolic
// ---------------------------------------------------------------------------
// node-pair keys are (lower << kb) | higher with kb the bits of the largest node index, so the radix sort
// runs over 2 kb bits only
__global__ void k_gen_pairs(int kind, const int32_t* __restrict__ n1, const int32_t* __restrict__ n2,
                            const int32_t* __restrict__ n3, const int32_t* __restrict__ n4, size_t begin,
                            size_t count, size_t pair_base, int kb, uint64_t* keys, uint32_t* vals) {
  size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k >= count) return;
  size_t e = begin + k;
  int ppe = kind == kPlate ? kPairs4 : kPairs2;
  int32_t nodes[4];
  nodes[0] = n1[e];
  nodes[1] = n2[e];
  if (kind == kPlate) {
    nodes[2] = n3[e];
    nodes[3] = n4[e];
  }
  for (int p = 0; p < ppe; ++p) {
    int i, j;
    if (kind == kPlate) pair_nodes4(p, i, j);
    else pair_nodes2(p, i, j);
    uint32_t I = (uint32_t)nodes[i], J = (uint32_t)nodes[j];
    uint32_t lo = I < J ? I : J, hi = I < J ? J : I;
    size_t pid = pair_base + k * ppe + p;
    keys[pid] = ((uint64_t)lo << kb) | hi;
    vals[pid] = ((uint32_t)kind << 30) | (uint32_t)(e * ppe + p);
  }
}

// v != 0.0 on the integer pipe (true for every value but +-0.0, NaN included):
// on GB300 an FP64 compare occupies the same narrow pipe as the arithmetic.
__device__ __forceinline__ bool nonzero(double v) { return (__double_as_longlong(v) << 1) != 0; }

// Packing of a block's entries in the scratch.  A global block whose every
// contribution is non-zero only inside the plate's structural set (membrane
// 2x2 u-v, plate 3x3 w-thx-thy and, on diagonal blocks, the drilling thz-thz:
// the shape of every flat-plate block, where R = I) stores 14 (diagonal) or 13
// (off-diagonal) entries per contribution in a fixed order; any other block
// stores all 36 row-major.  Both sets are closed under transposition.
enum : uint32_t { kLayFull = 0, kLayDiag14 = 1, kLayOff13 = 2 };
__constant__ int8_t c_lay_en[3][36] = {
    {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 17,
     18, 19, 20, 21, 22, 23, 24, 25, 26, 27, 28, 29, 30, 31, 32, 33, 34, 35},
    {0, 1, 6, 7, 14, 15, 16, 20, 21, 22, 26, 27, 28, 35},
    {0, 1, 6, 7, 14, 15, 16, 20, 21, 22, 26, 27, 28}};
constexpr uint64_t kSetOff13 = (1ull << 0) | (1ull << 1) | (1ull << 6) | (1ull << 7) | (1ull << 14) | (1ull << 15) |
                               (1ull << 16) | (1ull << 20) | (1ull << 21) | (1ull << 22) | (1ull << 26) |
                               (1ull << 27) | (1ull << 28);
constexpr uint64_t kSetDiag14 = kSetOff13 | (1ull << 35);
__host__ __device__ constexpr int lay_size(uint32_t lay) { return lay == kLayFull ? 36 : lay == kLayDiag14 ? 14 : 13; }
// doubles one contribution occupies: the 13-entry packing is padded to 14 (its 14th word holds the block's
// entry 35, which is zero for such a block), so every contribution starts on a 16-byte boundary and is
// written with 16-byte stores
__host__ __device__ constexpr int lay_stride(uint32_t lay) { return lay == kLayFull ? 36 : 14; }

// a 6x6 block in element orientation -> destination, transposed (to the
// block's (lower node, higher node) orientation) when the element's first node
// of the pair has the larger global index.
//   mask mode:    record the 36-bit mask of the block's non-zero entries;
//   numeric mode: write the block's packed entries at this contribution's
//                 offset in the scratch V (offset in the low 62 bits of
//                 pack[ep], packing in the top 2); a non-zero outside a
//                 structural packing raises *flag (the pattern changed).
struct BlockSink {
  uint64_t* mask;                       // mask mode: per (element, pair)
  double* V;                            // numeric mode
  const unsigned long long* pack;       // numeric mode: per (element, pair)
  int* flag;
  unsigned long long v_words = kNoBound;  // numeric mode: doubles of V (checked in debug builds)
  __device__ __forceinline__ void put(size_t ep, bool transpose, const double blk[36]) const {
    if (mask) {
      uint64_t m = 0;
#pragma unroll
      for (int a = 0; a < 6; ++a)
#pragma unroll
        for (int b = 0; b < 6; ++b) {
          int e = transpose ? 6 * b + a : 6 * a + b;
          if (nonzero(blk[6 * a + b])) m |= 1ull << e;
        }
      mask[ep] = m;
      return;
    }
    put_pk(pack[ep], transpose, blk);
  }
  // numeric mode, the pair's scratch position and layout word already read
  __device__ __forceinline__ void put_pk(unsigned long long pk, bool transpose, const double blk[36]) const {
    const uint32_t lay = (uint32_t)(pk >> 62);
    if (!dbg_in_range((pk & ((1ull << 62) - 1ull)) + (unsigned long long)lay_stride(lay) - 1ull, v_words, kDbgScratch))
      return;
    // 16-byte aligned: V is, and every contribution's offset is even
    double2* dst = reinterpret_cast<double2*>(V + (pk & ((1ull << 62) - 1ull)));
    if (lay == kLayFull) {
#pragma unroll
      for (int q = 0; q < 18; ++q) {
        const int e0 = 2 * q, e1 = 2 * q + 1;
        dst[q] = transpose ? make_double2(blk[6 * (e0 % 6) + e0 / 6], blk[6 * (e1 % 6) + e1 / 6])
                           : make_double2(blk[e0], blk[e1]);
      }
      return;
    }
    // structural packings: the set is symmetric, so a transposed block packs its
    // transposed entries at the same positions
    const int8_t order[14] = {0, 1, 6, 7, 14, 15, 16, 20, 21, 22, 26, 27, 28, 35};
    bool outside = false;
#pragma unroll
    for (int en = 0; en < 36; ++en) {
      bool in = (kSetOff13 >> en) & 1ull;
      if (!in && en != 35) outside |= nonzero(blk[en]);
    }
    double w[14];
#pragma unroll
    for (int j = 0; j < 14; ++j) {
      const int en = order[j];
      w[j] = transpose ? blk[6 * (en % 6) + en / 6] : blk[en];
    }
#pragma unroll
    for (int q = 0; q < 7; ++q) dst[q] = make_double2(w[2 * q], w[2 * q + 1]);
    if (lay != kLayDiag14) outside |= nonzero(blk[35]);
    if (outside) atomicOr(flag, 1);
  }
};

struct TrussView {
  const int32_t *n1, *n2;
  const double *E, *A, *A2;
};

__device__ __forceinline__ void truss_element(size_t e, NodesView nd, const TrussView& t, double abs_tol,
                                              const BlockSink& sink) {
  int I = t.n1[e], J = t.n2[e];
  double x1[3], x2[3], g[9];
  nd.get(I, x1);
  nd.get(J, x2);
  if (!truss_block(x1, x2, t.E[e], t.A[e], t.A2[e], abs_tol, g)) {
#pragma unroll
    for (int k = 0; k < 9; ++k) g[k] = 0.0;
  }
  double blk[36];
#pragma unroll
  for (int s = 0; s < 3; ++s) {
#pragma unroll
    for (int k = 0; k < 36; ++k) blk[k] = 0.0;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) blk[6 * a + b] = s == 1 ? -g[3 * a + b] : g[3 * a + b];
    sink.put(e * kPairs2 + s, s == 1 && I > J, blk);
  }
}

__global__ void __launch_bounds__(256) k_truss(NodesView nd, TrussView t, double abs_tol, size_t count,
                                               BlockSink sink) {
  size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= count) return;
  truss_element(e, nd, t, abs_tol, sink);
}

__device__ __forceinline__ void beam_element(size_t e, NodesView nd, const BeamView& b, double rel_tol,
                                             double abs_tol, const BlockSink& sink) {
  int I = b.n1[e], J = b.n2[e];
  double x1[3], x2[3];
  nd.get(I, x1);
  nd.get(J, x2);
  double axis[3] = {b.ax[e], b.ay[e], b.az[e]};
  BeamBlocks B;
  if (!beam_blocks(x1, x2, b.E[e], b.nu[e], b.A[e], b.i11[e], b.i22[e], b.i12[e], b.it[e], b.ks[e], axis, rel_tol,
                   abs_tol, B)) {
#pragma unroll
    for (int k = 0; k < 9; ++k) B.uu[k] = B.ut[k] = B.th[k] = B.tu[k] = B.thth2[k] = 0.0;
  }
  double blk[36];
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
  sink.put(e * kPairs2 + 0, false, blk);
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
  sink.put(e * kPairs2 + 1, I > J, blk);
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
  sink.put(e * kPairs2 + 2, false, blk);
}

__global__ void __launch_bounds__(256) k_beam(NodesView nd, BeamView b, double rel_tol, double abs_tol, size_t count,
                                              BlockSink sink) {
  size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= count) return;
  beam_element(e, nd, b, rel_tol, abs_tol, sink);
}

// node pair P = (I, J) of the plate; its scratch word comes from spk[P * spk_stride] when the caller staged the
// plate's words in shared memory, else from the sink's array.  IDENT (R = I) is a template argument so that the
// identity path keeps the local block's structural zeros as compile-time zeros (no rotation, no merge with the
// rotated values, no run-time tests of entries known to be zero).
template <int I, int J, int P, bool IDENT>
__device__ __forceinline__ void plate_pair(const PlateCore& C, const double R[9], const int nidx[4], size_t e,
                                           const BlockSink& sink, const unsigned long long* spk, unsigned spk_stride) {
  double blk[36];
  plate_block_ct<I, J>(C, blk);
  if constexpr (!IDENT) {
    double o[36];
    plate_rotate_block_ct<I == J>(R, blk, o);
#pragma unroll
    for (int k = 0; k < 36; ++k) blk[k] = o[k];
  }
  const bool transpose = I != J && nidx[I] > nidx[J];
  if (spk)
    sink.put_pk(spk[P * spk_stride], transpose, blk);
  else
    sink.put(e * kPairs4 + P, transpose, blk);
}

// the ten node pairs in the order of pair_nodes4
template <bool IDENT>
__device__ __forceinline__ void plate_pairs(const PlateCore& C, const double R[9], const int nidx[4], size_t e,
                                            const BlockSink& sink, const unsigned long long* spk, unsigned stride) {
  plate_pair<0, 0, 0, IDENT>(C, R, nidx, e, sink, spk, stride);
  plate_pair<0, 1, 1, IDENT>(C, R, nidx, e, sink, spk, stride);
  plate_pair<0, 2, 2, IDENT>(C, R, nidx, e, sink, spk, stride);
  plate_pair<0, 3, 3, IDENT>(C, R, nidx, e, sink, spk, stride);
  plate_pair<1, 1, 4, IDENT>(C, R, nidx, e, sink, spk, stride);
  plate_pair<1, 2, 5, IDENT>(C, R, nidx, e, sink, spk, stride);
  plate_pair<1, 3, 6, IDENT>(C, R, nidx, e, sink, spk, stride);
  plate_pair<2, 2, 7, IDENT>(C, R, nidx, e, sink, spk, stride);
  plate_pair<2, 3, 8, IDENT>(C, R, nidx, e, sink, spk, stride);
  plate_pair<3, 3, 9, IDENT>(C, R, nidx, e, sink, spk, stride);
}

// 8-byte asynchronous copy global -> shared (each thread copies only words it reads itself, so waiting for its
// own copies is enough: no barrier)
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

__device__ __forceinline__ void plate_element(size_t e, NodesView nd, const PlateView& pl, double abs_tol,
                                              const BlockSink& sink, const unsigned long long* spk = nullptr,
                                              unsigned spk_stride = 0) {
  int nidx[4] = {pl.n1[e], pl.n2[e], pl.n3[e], pl.n4[e]};
  double X[4][3];
#pragma unroll
  for (int k = 0; k < 4; ++k) nd.get(nidx[k], X[k]);
  double R[9];
  if (!plate_rotation(X[1], X[2], X[3], abs_tol, R)) set_identity(R);
  const bool ident = is_identity(R);
  double xl[4], yl[4];
  plate_local_xy(X, R, ident, xl, yl);
  PlateCore C;
  plate_core(xl, yl, pl.E[e], pl.nu[e], pl.t[e], pl.ks[e], C);
  if (spk) cp_async_wait_all();
  if (ident)
    plate_pairs<true>(C, R, nidx, e, sink, spk, spk_stride);
  else
    plate_pairs<false>(C, R, nidx, e, sink, spk, spk_stride);
}

// Launch shape of the plate kernel.  FEM_PLATE_BLOCK threads per CTA (64 by default) and at most
// FEM_PLATE_MAXNREG registers a thread (200 by default: five 64-thread CTAs, 10 warps, an SM instead of
// four at the 254 the kernel takes uncapped; the 160 bytes a thread spills cost less than the two warps
// win -- 1.0185 against 1.0226 ms on the 1M-plate mesh; caps of 168 and 128 were no better or slower).
#ifndef FEM_PLATE_BLOCK
#define FEM_PLATE_BLOCK 64
#endif
#ifndef FEM_PLATE_MAXNREG
#define FEM_PLATE_MAXNREG 200
#endif
__global__ void __maxnreg__(FEM_PLATE_MAXNREG)
k_plate(NodesView nd, PlateView pl, double abs_tol, size_t count,
                                               BlockSink sink) {
  // numeric mode: the plate's ten scratch words are copied to shared memory ([pair][thread], dynamic, sized
  // kPairs4 x blockDim.x by plate_smem) while the element arithmetic runs, instead of being loaded at each store
  extern __shared__ unsigned long long s_pack[];
  size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= count) return;
  const unsigned long long* spk = nullptr;
  if (sink.pack) {
#pragma unroll
    for (int p = 0; p < kPairs4; ++p) cp_async8(&s_pack[p * blockDim.x + threadIdx.x], sink.pack + e * kPairs4 + p);
    cp_async_commit();
    spk = &s_pack[threadIdx.x];
  }
  plate_element(e, nd, pl, abs_tol, sink, spk, blockDim.x);
}
// dynamic shared memory of a k_plate launch of `block` threads
size_t plate_smem(const BlockSink& sink, unsigned block) {
  return sink.pack ? (size_t)kPairs4 * block * sizeof(unsigned long long) : 0;
}

// sorted position k: record the element pair's slot and its mask
__global__ void k_scatter_slots(const uint32_t* __restrict__ vals, size_t n, uint32_t* slot_t, uint32_t* slot_b,
                                uint32_t* slot_p, const uint64_t* mask_t, const uint64_t* mask_b,
                                const uint64_t* mask_p, uint64_t* sorted_mask) {
  size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  uint32_t v = vals[k];
  uint32_t kind = v >> 30, idx = v & 0x3fffffffu;
  uint32_t* s = kind == kTruss ? slot_t : kind == kBeam ? slot_b : slot_p;
  const uint64_t* m = kind == kTruss ? mask_t : kind == kBeam ? mask_b : mask_p;
  s[idx] = (uint32_t)k;
  sorted_mask[k] = m[idx];
}

__global__ void k_heads(const uint64_t* __restrict__ keys, size_t n, uint32_t* head) {
  size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  head[k] = (k == 0 || keys[k] != keys[k - 1]) ? 1u : 0u;
}

// blk_id = inclusive scan of heads - 1
__global__ void k_block_starts(const uint32_t* __restrict__ blk_incl, size_t n, uint32_t* blk_start) {
  size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  if (k == 0 || blk_incl[k] != blk_incl[k - 1]) blk_start[blk_incl[k] - 1] = (uint32_t)k;
}

__device__ __forceinline__ uint64_t transpose36(uint64_t m) {
  uint64_t t = 0;
  for (int a = 0; a < 6; ++a)
    for (int b = 0; b < 6; ++b)
      if ((m >> (6 * a + b)) & 1ull) t |= 1ull << (6 * b + a);
  return t;
}

__global__ void k_block_meta(const uint32_t* __restrict__ blk_start, size_t nb, size_t n_pairs,
                             const uint64_t* __restrict__ keys, int kb, const uint64_t* __restrict__ sorted_mask,
                             uint32_t* blk_count, uint64_t* blk_mask, uint64_t* blk_maskT, int32_t* blk_I,
                             int32_t* blk_J) {
  size_t b = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (b >= nb) return;
  uint32_t s = blk_start[b];
  uint32_t e = b + 1 < nb ? blk_start[b + 1] : (uint32_t)n_pairs;
  uint64_t m = 0;
  for (uint32_t k = s; k < e; ++k) m |= sorted_mask[k];
  blk_count[b] = e - s;
  blk_mask[b] = m;
  blk_maskT[b] = transpose36(m);
  uint64_t key = keys[s];
  int32_t I = (int32_t)(key >> kb), J = (int32_t)(key & ((1ull << kb) - 1ull));
  blk_I[b] = I;
  blk_J[b] = J;
}

// Row-node adjacency from the blocks, which are in (I, J) order with I <= J: row r lists the blocks (I, r),
// I <= r, in I order (a stable sort of the blocks by J) and then the blocks (r, J), J > r, in J order (a
// range of the block order) -- the (row node, column node) order without sorting on both nodes.
__global__ void k_block_cols(size_t nb, const int32_t* __restrict__ blk_J, uint32_t* col, uint32_t* idx) {
  const size_t b = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (b >= nb) return;
  col[b] = (uint32_t)blk_J[b];
  idx[b] = (uint32_t)b;
}
// first and end position of every key's run in a sorted array (untouched for keys absent)
template <class K>
__global__ void k_runs(const K* __restrict__ keys, size_t n, int32_t* first, int32_t* end) {
  const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t r = (uint32_t)keys[k];
  if (k == 0 || (uint32_t)keys[k - 1] != r) first[r] = (int32_t)k;
  if (k + 1 == n || (uint32_t)keys[k + 1] != r) end[r] = (int32_t)(k + 1);
}
// entries of row r: its column run (blocks (I, r)) and its row run past the diagonal (blocks (r, J), J > r)
__device__ __forceinline__ void adj_parts(size_t r, const int32_t* jf, const int32_t* je, const int32_t* i_f,
                                          const int32_t* ie, const int32_t* __restrict__ blk_J, int32_t& n_low,
                                          int32_t& up_first, int32_t& n_up) {
  n_low = jf[r] >= 0 ? je[r] - jf[r] : 0;
  up_first = i_f[r];
  n_up = 0;
  if (up_first >= 0) {
    n_up = ie[r] - up_first;
    if (blk_J[up_first] == (int32_t)r) {  // the diagonal block leads the row run; it is in the column run
      ++up_first;
      --n_up;
    }
  }
}
__global__ void k_adj_lens(size_t nn, const int32_t* jf, const int32_t* je, const int32_t* i_f, const int32_t* ie,
                           const int32_t* __restrict__ blk_J, uint32_t* len) {
  const size_t r = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (r > nn) return;
  if (r == nn) {
    len[r] = 0;
    return;
  }
  int32_t n_low, up_first, n_up;
  adj_parts(r, jf, je, i_f, ie, blk_J, n_low, up_first, n_up);
  len[r] = (uint32_t)(n_low + n_up);
}
__global__ void k_adj_fill(size_t nn, const int32_t* jf, const int32_t* je, const int32_t* i_f, const int32_t* ie,
                           const int32_t* __restrict__ blk_I, const int32_t* __restrict__ blk_J,
                           const uint32_t* __restrict__ by_col, const uint32_t* __restrict__ off, int kb,
                           uint64_t* akeys, uint32_t* avals, int32_t* seg_begin, int32_t* seg_end) {
  const size_t r = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (r >= nn) return;
  int32_t n_low, up_first, n_up;
  adj_parts(r, jf, je, i_f, ie, blk_J, n_low, up_first, n_up);
  const uint32_t o = off[r];
  seg_begin[r] = n_low + n_up > 0 ? (int32_t)o : -1;
  seg_end[r] = n_low + n_up > 0 ? (int32_t)(o + n_low + n_up) : -1;
  for (int32_t k = 0; k < n_low; ++k) {
    const uint32_t b = by_col[jf[r] + k];
    const uint32_t I = (uint32_t)blk_I[b];
    akeys[o + k] = ((uint64_t)r << kb) | I;
    avals[o + k] = (b << 1) | (I != (uint32_t)r ? 1u : 0u);
  }
  for (int32_t k = 0; k < n_up; ++k) {
    const uint32_t b = (uint32_t)(up_first + k);
    akeys[o + n_low + k] = ((uint64_t)r << kb) | (uint32_t)blk_J[b];
    avals[o + n_low + k] = b << 1;
  }
}

__device__ __forceinline__ uint32_t kinds_of(uint64_t m) {
  const uint64_t q0 = 0x1c71c7ull;        // rows 0-2, cols 0-2
  const uint64_t q1 = q0 << 3;            // rows 0-2, cols 3-5
  const uint64_t q2 = q0 << 18;           // rows 3-5, cols 0-2
  const uint64_t q3 = q0 << 21;           // rows 3-5, cols 3-5
  return ((m & q0) ? 1u : 0u) | ((m & q1) ? 2u : 0u) | ((m & q2) ? 4u : 0u) | ((m & q3) ? 8u : 0u);
}

// per row node: the lengths of its 6 rows and its group count
__global__ void k_row_counts(size_t n_nodes, const int32_t* __restrict__ seg_begin,
                             const int32_t* __restrict__ seg_end, const uint32_t* __restrict__ avals,
                             const uint64_t* __restrict__ blk_mask, const uint64_t* __restrict__ blk_maskT,
                             int64_t* row_nnz, int64_t* gcount) {
  size_t r = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (r >= n_nodes) return;
  int32_t run[6] = {0, 0, 0, 0, 0, 0};
  int64_t ng = 0;
  int32_t s = seg_begin[r], e = seg_end[r];
  for (int32_t k = s; k < e && s >= 0; ++k) {
    uint32_t v = avals[k];
    uint32_t b = v >> 1, t = v & 1u;
    uint64_t m = t ? blk_maskT[b] : blk_mask[b];
    for (int a = 0; a < 6; ++a) run[a] += __popcll((m >> (6 * a)) & 63ull);
    ng += __popc(kinds_of(m));
  }
  for (int a = 0; a < 6; ++a) row_nnz[6 * r + a] = run[a];
  gcount[r] = ng;
}

// ---------------------------------------------------------------------------
// compacted scratch layout
// ---------------------------------------------------------------------------
// Block b stores count_b contributions of lay_stride(layout_b) doubles each,
// contiguous and in element order, at blk_voff[b] (an exclusive scan of
// count_b * lay_stride).
__global__ void k_block_sizes(size_t nb, const uint32_t* __restrict__ blk_count, const uint64_t* __restrict__ blk_mask,
                              const int32_t* __restrict__ blk_I, const int32_t* __restrict__ blk_J, uint8_t* blk_lay,
                              uint64_t* blk_pmask, unsigned long long* sizes, unsigned long long* pad_words) {
  const size_t b = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  unsigned pad = 0;
  if (b < nb) {
    const uint64_t m = blk_mask[b];
    uint32_t lay = kLayFull;
    if (blk_I[b] == blk_J[b]) {
      if ((m & ~kSetDiag14) == 0) lay = kLayDiag14;
    } else if ((m & ~kSetOff13) == 0) {
      lay = kLayOff13;
    }
    blk_lay[b] = (uint8_t)lay;
    // the pattern over packed positions: bit j set when packed entry j is a pattern entry
    uint64_t pm = 0;
    for (int j = 0; j < lay_size(lay); ++j)
      if ((m >> c_lay_en[lay][j]) & 1ull) pm |= 1ull << j;
    blk_pmask[b] = pm;
    sizes[b] = (unsigned long long)blk_count[b] * (unsigned long long)lay_stride(lay);
    pad = (unsigned)(lay_stride(lay) - lay_size(lay)) * blk_count[b];
  }
  // padding words of the CTA's blocks, one atomic per CTA (blockDim.x = 256)
  __shared__ unsigned long long warp_pad[8];
  const unsigned wsum = __reduce_add_sync(0xffffffffu, pad);
  if ((threadIdx.x & 31) == 0) warp_pad[threadIdx.x >> 5] = wsum;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += warp_pad[w];
    if (t) atomicAdd(pad_words, t);
  }
}

// per element pair: its packed offset in V (low 62 bits) and the block's packing (top 2 bits)
__global__ void k_pair_offsets(const uint32_t* __restrict__ svals, const uint32_t* __restrict__ incl, size_t n,
                               const uint32_t* __restrict__ blk_start, const unsigned long long* __restrict__ blk_voff,
                               const uint8_t* __restrict__ blk_lay, unsigned long long* pk_t,
                               unsigned long long* pk_b, unsigned long long* pk_p) {
  size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  uint32_t v = svals[k];
  uint32_t kind = v >> 30, idx = v & 0x3fffffffu;
  uint32_t b = incl[k] - 1;
  const uint32_t lay = blk_lay[b];
  unsigned long long off = blk_voff[b] + (unsigned long long)(k - blk_start[b]) * (unsigned long long)lay_stride(lay);
  off |= (unsigned long long)lay << 62;
  if (kind == kTruss) pk_t[idx] = off;
  else if (kind == kBeam) pk_b[idx] = off;
  else pk_p[idx] = off;
}

// ---------------------------------------------------------------------------
// kernel: deterministic block reduction into CSR
// ---------------------------------------------------------------------------
constexpr int kFlagPattern = 1;                      // bit of *flag: the exact-zero pattern changed

// Block-sum slots.  A packed entry of a block with one contribution needs no
// sum: its CSR value is gathered straight from the scratch.  Entries of blocks
// with 2, 3, 4 and 5+ contributions get a slot in S, grouped by that count so a
// warp adds the same number of terms on every lane (on GB300 the FP64 adds of
// the reduction are themselves a throughput limit).  Blocks with one
// contribution keep a check-only descriptor for each packed entry outside the
// pattern (to see the exact-zero pattern change).  Categories: 0 = one
// contribution, 1..4 = 2, 3, 4, 5+ contributions.
constexpr int kSlotCats = 5;
__host__ __device__ __forceinline__ int slot_cat(uint32_t count) { return count <= 1 ? 0 : count >= 5 ? 4 : (int)count - 1; }

__global__ void k_slot_sizes(size_t nb, const uint32_t* __restrict__ blk_count, const uint64_t* __restrict__ blk_pmask,
                             const uint8_t* __restrict__ blk_lay, unsigned long long* sz /* kSlotCats x (nb + 1) */) {
  size_t b = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (b >= nb) return;
  const int c = lay_size(blk_lay[b]);
  const int cat = slot_cat(blk_count[b]);
#pragma unroll
  for (int g = 0; g < kSlotCats; ++g) sz[(size_t)g * (nb + 1) + b] = 0;
  sz[(size_t)cat * (nb + 1) + b] = cat == 0 ? (unsigned long long)(c - __popcll(blk_pmask[b])) : (unsigned long long)c;
}

struct SlotLayout {
  const unsigned long long* base;  // kSlotCats x (nb + 1): per category, exclusive scan over blocks
  size_t stride;                   // nb + 1
  unsigned long long off[kSlotCats];  // first descriptor of each category (category 0 last)
  unsigned long long vs_off;          // S starts at this scratch position
};

// position of a block entry in its packing (-1: not packed)
// (the packed entries are listed in ascending entry order, so the position is the number of set entries below)
__device__ __forceinline__ int packed_pos(uint32_t lay, int en) {
  if (lay == kLayFull) return en;
  const uint64_t set = lay == kLayDiag14 ? kSetDiag14 : kSetOff13;
  return ((set >> en) & 1ull) ? __popcll(set & ((1ull << en) - 1ull)) : -1;
}

// inclusive prefix sum over the lanes of a warp
constexpr int kRowLanes = 16;  // lanes per node in the row fill (a plate-mesh node has 9 blocks, a frame node 7)

// inclusive prefix sum over the kRowLanes lanes of a node
__device__ __forceinline__ int seg_inclusive_sum(int v) {
  const int sl = threadIdx.x & (kRowLanes - 1);
#pragma unroll
  for (int d = 1; d < kRowLanes; d <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, v, d, kRowLanes);
    if (sl >= d) v += u;
  }
  return v;
}

// Symbolic, once per pattern: the CSR rows of a node, kRowLanes lanes per node.
// Lane k takes the k-th block of the node's adjacency (blocks in column-node
// order, kRowLanes at a time); for each of the node's 6 rows a prefix sum of the
// blocks' entry counts gives every lane the place of its entries, which it
// writes in column order: column, stiffness group and value source (the
// scratch position of a block with one contribution, else the entry's
// block-sum slot in S -- both in one buffer, S starting at vs_off).  A block
// stored with the row node second (t = 1) is read transposed.  The node's
// groups are placed the same way.
__global__ void k_row_fill(size_t node0, size_t n_nodes, const int32_t* __restrict__ seg_begin, const int32_t* __restrict__ seg_end,
                           const uint64_t* __restrict__ akeys, int kb, const uint32_t* __restrict__ avals,
                           const uint64_t* __restrict__ blk_mask, const uint64_t* __restrict__ blk_maskT,
                           const uint8_t* __restrict__ blk_lay, const uint32_t* __restrict__ blk_count,
                           const unsigned long long* __restrict__ blk_voff, SlotLayout L,
                           const int64_t* __restrict__ row_ptr, const int64_t* __restrict__ gbase,
                           int32_t* __restrict__ col_idx, int32_t* __restrict__ nnz_group,
                           uint32_t* __restrict__ src_map, int32_t* __restrict__ g_row, int32_t* __restrict__ g_col,
                           uint8_t* __restrict__ g_kind, unsigned long long nnz, unsigned long long n_groups,
                           unsigned long long vs_end) {
  const size_t r = node0 + (blockIdx.x * (size_t)blockDim.x + threadIdx.x) / kRowLanes;
  const int lane = (int)(threadIdx.x & (kRowLanes - 1));
  // every lane stays for the shuffles: a node past the end or without blocks has an empty range
  int32_t s = 0, e = 0;
  if (r < n_nodes && seg_begin[r] >= 0) {
    s = seg_begin[r];
    e = seg_end[r];
  }
  int64_t gnext = 0;
  int64_t next[6] = {0, 0, 0, 0, 0, 0};
  if (e > s) {
    gnext = gbase[r];
#pragma unroll
    for (int a = 0; a < 6; ++a) next[a] = row_ptr[6 * r + a];
  }
  for (int32_t k0 = s; __any_sync(0xffffffffu, k0 < e); k0 += kRowLanes) {
    const int32_t k = k0 + lane;
    uint64_t m = 0;
    uint32_t J = 0, lay = 0, t = 0;
    unsigned long long sb = 0;
    if (k < e) {
      const uint32_t v = avals[k];
      const uint32_t b = v >> 1;
      t = v & 1u;
      J = (uint32_t)(akeys[k] & ((1ull << kb) - 1ull));
      m = t ? blk_maskT[b] : blk_mask[b];
      lay = blk_lay[b];
      const int cat = slot_cat(blk_count[b]);
      sb = cat == 0 ? blk_voff[b] : L.vs_off + L.off[cat] + L.base[(size_t)cat * L.stride + b];
    }
    // groups
    const uint32_t km = kinds_of(m);
    const int ng = __popc(km);
    const int gin = seg_inclusive_sum(ng);
    int64_t g = gnext + gin - ng;
    int32_t kg[4];
#pragma unroll
    for (int kd = 0; kd < 4; ++kd) {
      kg[kd] = -1;
      if (km & (1u << kd)) {
        if (dbg_in_range((unsigned long long)g, n_groups, kDbgGroup)) {
          g_row[g] = (int32_t)r;
          g_col[g] = (int32_t)J;
          g_kind[g] = (uint8_t)kd;
        }
        kg[kd] = (int32_t)g;
        ++g;
      }
    }
    gnext += __shfl_sync(0xffffffffu, gin, kRowLanes - 1, kRowLanes);
    // rows
#pragma unroll
    for (int a = 0; a < 6; ++a) {
      const uint32_t rowbits = (uint32_t)((m >> (6 * a)) & 63ull);
      const int cnt = __popc(rowbits);
      const int inc = seg_inclusive_sum(cnt);
      int64_t pos = next[a] + inc - cnt;
#pragma unroll
      for (int c = 0; c < 6; ++c)
        if (rowbits & (1u << c)) {
          const unsigned long long src = sb + (unsigned long long)packed_pos(lay, t ? 6 * c + a : 6 * a + c);
          if (dbg_in_range((unsigned long long)pos, nnz, kDbgCsrEntry) && dbg_in_range(src, vs_end, kDbgRowSource)) {
            col_idx[pos] = (int32_t)(6 * J + c);
            nnz_group[pos] = kg[2 * (a / 3) + c / 3];
            src_map[pos] = (uint32_t)src;
          }
          ++pos;
        }
      next[a] += __shfl_sync(0xffffffffu, inc, kRowLanes - 1, kRowLanes);
    }
  }
}

// Symbolic, once per pattern: the descriptors -- the scratch position of the
// first contribution, the number of contributions (bits 0-23), the stride
// between contributions (bits 24-30: lay_stride), and whether
// the entry is a pattern entry (bit 31).
__global__ void k_slot_desc(size_t nb, const uint32_t* __restrict__ blk_count, const uint64_t* __restrict__ blk_pmask,
                            const uint8_t* __restrict__ blk_lay, const unsigned long long* __restrict__ blk_voff,
                            SlotLayout L, uint2* desc, int* too_many) {
  const size_t b = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (b >= nb) return;
  const int c = lay_size(blk_lay[b]);
  const uint32_t cnt = blk_count[b];
  if (cnt >= (1u << 24)) atomicOr(too_many, 1);
  const uint64_t pm = blk_pmask[b];
  const int cat = slot_cat(cnt);
  const unsigned long long voff = blk_voff[b];
  const uint32_t hi = (cnt & 0xffffffu) | ((uint32_t)lay_stride(blk_lay[b]) << 24);
  if (cat == 0) {
    // one contribution: pattern entries are gathered straight from the scratch; the others get a check
    unsigned long long at = L.off[0] + L.base[b];
    for (int j = 0; j < c; ++j)
      if (!((pm >> j) & 1ull)) desc[at++] = make_uint2((uint32_t)(voff + (unsigned long long)j), hi);
  } else {
    const unsigned long long at = L.off[cat] + L.base[(size_t)cat * L.stride + b];
    for (int j = 0; j < c; ++j)
      desc[at + j] = make_uint2((uint32_t)(voff + (unsigned long long)j), hi | ((uint32_t)((pm >> j) & 1ull) << 31));
  }
}

// Numeric pass, part 1: one thread per descriptor.  Slots in S (descriptors
// below n_sums) sum their contributions in element order (left to right, as
// the reference's call-order accumulation): descriptors are grouped by
// contribution count, so every lane of a warp adds the same number of terms.
// Check-only descriptors (one contribution, outside the pattern) only test
// their entry.  No atomics on values.  A non-pattern entry with a non-zero, or
// a pattern slot whose contributions are all zero, raises kFlagPattern (the
// exact-zero pattern changed).
__device__ __forceinline__ bool block_sum_one(size_t i, uint2 d, size_t n_sums, const double* __restrict__ V,
                                              double* __restrict__ S, unsigned long long v_words) {
  const uint32_t n = d.y & 0xffffffu, stride = (d.y >> 24) & 0x7fu;
  const bool inpat = (d.y >> 31) != 0;
  if (n == 0 || !dbg_in_range(d.x + (unsigned long long)(n - 1) * stride, v_words, kDbgSumSource)) return false;
  const double* src = V + d.x;
  bool nz;
  double sum;
  switch (n) {
    case 1:
      return nonzero(src[0]);
    case 2: {
      const double a = src[0], b = src[stride];
      nz = nonzero(a) | nonzero(b);
      sum = a + b;
      break;
    }
    case 3: {
      const double a = src[0], b = src[stride], c = src[2 * stride];
      nz = nonzero(a) | nonzero(b) | nonzero(c);
      sum = (a + b) + c;
      break;
    }
    case 4: {
      const double a = src[0], b = src[stride], c = src[2 * stride], e = src[3 * stride];
      nz = nonzero(a) | nonzero(b) | nonzero(c) | nonzero(e);
      sum = ((a + b) + c) + e;
      break;
    }
    default: {
      sum = src[0];
      nz = nonzero(sum);
      for (uint32_t k = 1; k < n; ++k) {
        const double x = src[(size_t)k * stride];
        nz |= nonzero(x);
        sum = sum + x;
      }
    }
  }
  if (i < n_sums) S[i] = sum;
  return nz != inpat;
}

// grid-stride over the descriptors, the next descriptor loaded while the current one's contributions are read
__global__ void __launch_bounds__(512) k_block_sums(size_t n_desc, size_t n_sums, const uint2* __restrict__ desc,
                                                    const double* __restrict__ V, double* __restrict__ S, int* flag,
                                                    unsigned long long v_words) {
  const size_t step = (size_t)gridDim.x * blockDim.x;
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n_desc) return;
  uint2 d = desc[i];
  bool bad = false;
  for (;;) {
    const size_t inext = i + step;
    const uint2 dn = inext < n_desc ? desc[inext] : make_uint2(0u, 0u);
    bad |= block_sum_one(i, d, n_sums, V, S, v_words);
    if (inext >= n_desc) break;
    i = inext;
    d = dn;
  }
  if (bad) atomicOr(flag, kFlagPattern);
}
// CTAs of a block-sum launch: enough to fill the SMs a few times over, each looping over its share
unsigned block_sums_grid(size_t n_desc, unsigned block) {
  static std::atomic<int> sms[64];  // per device, 0 = not asked yet (calls may come from several threads)
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) dev = 0;
  int n = sms[dev].load(std::memory_order_relaxed);
  if (!n) {
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) n = 1;
    sms[dev].store(n, std::memory_order_relaxed);
  }
  const size_t want = (n_desc + block - 1) / block, cap = (size_t)n * (2048 / block) * 2;
  return (unsigned)std::max<size_t>(1, std::min(want, cap));
}

// Numeric pass, part 2: CSR values in storage order, each read from its source
// (the scratch for one-contribution entries, S otherwise; S starts at vs_off of
// the same buffer).  A warp takes 32 x kGatherPerThread consecutive entries and
// lane t entries t, t + 32, ...: every load of the source map and every store of
// the values is one contiguous warp access, and neighbouring entries of a row
// (neighbouring sources) sit in neighbouring lanes.  A one-contribution pattern
// entry that reads zero raises kFlagPattern.
constexpr int kGatherPerThread = 8;
__global__ void __launch_bounds__(512) k_gather_values(size_t nnz, const uint32_t* __restrict__ src_map,
                                                       const double* __restrict__ VS, unsigned long long vs_off,
                                                       double* __restrict__ values, int* flag,
                                                       unsigned long long vs_end) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t k0 = (t >> 5) * (32 * kGatherPerThread) + (t & 31);
  if (k0 >= nnz) return;
  bool zero_direct = false;
  uint32_t sx[kGatherPerThread];
#pragma unroll
  for (int q = 0; q < kGatherPerThread; ++q) {
    const size_t k = k0 + 32 * (size_t)q;
    sx[q] = k < nnz ? src_map[k] : 0u;
  }
  double a[kGatherPerThread];
#pragma unroll
  for (int q = 0; q < kGatherPerThread; ++q)
    a[q] = (k0 + 32 * (size_t)q < nnz && dbg_in_range(sx[q], vs_end, kDbgGatherSource)) ? VS[sx[q]] : 0.0;
#pragma unroll
  for (int q = 0; q < kGatherPerThread; ++q) {
    const size_t k = k0 + 32 * (size_t)q;
    if (k < nnz) {
      zero_direct |= sx[q] < vs_off && !nonzero(a[q]);
      values[k] = a[q];
    }
  }
  if (zero_direct) atomicOr(flag, kFlagPattern);
}

// ---------------------------------------------------------------------------
// host helpers
// ---------------------------------------------------------------------------
// Rust's {:?} for f64 (shortest round-trip digits; plain notation for
// 1e-4 <= |v| < 1e16, else d.ddde[-]x)
std::string rust_f64(double v) {
  if (v != v) return "NaN";
  if (std::isinf(v)) return v > 0 ? "inf" : "-inf";
  if (v == 0.0) return std::signbit(v) ? "-0.0" : "0.0";
  char buf[64];
  for (int prec = 1; prec <= 17; ++prec) {
    snprintf(buf, sizeof buf, "%.*e", prec - 1, v);
    if (strtod(buf, nullptr) == v) break;
  }
  std::string s(buf);
  size_t epos = s.find('e');
  int ex = atoi(s.c_str() + epos + 1);
  std::string mant = s.substr(0, epos);
  bool neg = mant[0] == '-';
  std::string digs;
  for (char c : mant)
    if (c >= '0' && c <= '9') digs.push_back(c);
  double av = std::fabs(v);
  std::string out = neg ? "-" : "";
  if (av >= 1e-4 && av < 1e16) {
    if (ex >= 0) {
      for (int i = 0; i <= ex; ++i) out.push_back(i < (int)digs.size() ? digs[i] : '0');
      out.push_back('.');
      if (ex + 1 < (int)digs.size()) out += digs.substr(ex + 1);
      else out.push_back('0');
    } else {
      out += "0.";
      for (int i = 0; i < -ex - 1; ++i) out.push_back('0');
      out += digs;
    }
  } else {
    while (digs.size() > 1 && digs.back() == '0') digs.pop_back();
    out.push_back(digs[0]);
    if (digs.size() > 1) {
      out.push_back('.');
      out += digs.substr(1);
    }
    out += "e" + std::to_string(ex);
  }
  return out;
}

struct CoordKey {
  uint64_t a, b, c;
  bool operator==(const CoordKey& o) const { return a == o.a && b == o.b && c == o.c; }
};
CoordKey coord_key(double x, double y, double z) {
  if (x == 0.0) x = 0.0;
  if (y == 0.0) y = 0.0;
  if (z == 0.0) z = 0.0;
  CoordKey k;
  memcpy(&k.a, &x, 8);
  memcpy(&k.b, &y, 8);
  memcpy(&k.c, &z, 8);
  return k;
}

uint64_t pair_key(uint32_t a, uint32_t b) {
  uint32_t lo = a < b ? a : b, hi = a < b ? b : a;
  return ((uint64_t)lo << 32) | hi;
}

struct Set4 {
  uint32_t s[4];
  bool operator==(const Set4& o) const { return !memcmp(s, o.s, sizeof s); }
};
// the four numbers in ascending order (a five-comparator sorting network)
Set4 sorted4(const uint32_t n[4]) {
  uint32_t a = n[0], b = n[1], c = n[2], d = n[3], t;
#define FEM_CSWAP(x, y) \
  if (y < x) {          \
    t = x;              \
    x = y;              \
    y = t;              \
  }
  FEM_CSWAP(a, b)
  FEM_CSWAP(c, d)
  FEM_CSWAP(a, c)
  FEM_CSWAP(b, d)
  FEM_CSWAP(b, c)
#undef FEM_CSWAP
  Set4 k;
  k.s[0] = a;
  k.s[1] = b;
  k.s[2] = c;
  k.s[3] = d;
  return k;
}

struct Run {
  int kind;
  size_t begin, count, pair_base;
};

uint64_t mix64(uint64_t x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ull;
  x ^= x >> 33;
  return x;
}

// A std::vector whose resize leaves new elements default-initialised (no zero fill), so that the
// first touch of a large host array happens in the threads that write it.
template <class T>
struct NoInitAlloc : std::allocator<T> {
  template <class U>
  struct rebind {
    using other = NoInitAlloc<U>;
  };
  NoInitAlloc() = default;
  template <class U>
  NoInitAlloc(const NoInitAlloc<U>&) {}
  template <class U>
  void construct(U* p) noexcept {
    ::new ((void*)p) U;
  }
  template <class U, class... A>
  void construct(U* p, A&&... a) {
    ::new ((void*)p) U(std::forward<A>(a)...);
  }
};
template <class T>
using HostVec = std::vector<T, NoInitAlloc<T>>;

// Open-addressing table of (64-bit key, value) with linear probing and
// backward-shift deletion; several entries may share a key (the caller's
// predicate tells them apart), so it serves as map, set and multimap.  The
// registries behind add_node / add_* (duplicate numbers, node pairs, plate
// node sets, exact coordinates) hold one entry per node or element.  Key and
// value share a 16-byte slot (one cache line touch per probe), the load stays
// at most 5/8, and bulk callers prefetch the home slot of an entry a few
// iterations ahead.
class FlatTable {
 public:
  FlatTable() { init(64); }
  template <class Eq>
  int64_t find(uint64_t key, Eq eq) const {
    size_t i = mix64(key) & mask_;
    while (slot_[i].val >= 0) {
      if (slot_[i].key == key && eq(slot_[i].val)) return slot_[i].val;
      i = (i + 1) & mask_;
    }
    return -1;
  }
  int64_t find(uint64_t key) const {
    return find(key, [](int64_t) { return true; });
  }
  void prefetch(uint64_t key) const { __builtin_prefetch(&slot_[mix64(key) & mask_]); }
  void insert(uint64_t key, int64_t v) {
    if (8 * (len_ + 1) > 5 * slot_.size()) rehash(slot_.size());
    put(key, v);
  }
  void erase(uint64_t key, int64_t v) {
    size_t i = mix64(key) & mask_;
    while (slot_[i].val >= 0 && !(slot_[i].key == key && slot_[i].val == v)) i = (i + 1) & mask_;
    if (slot_[i].val < 0) return;
    // backward-shift deletion
    size_t j = i;
    for (;;) {
      j = (j + 1) & mask_;
      if (slot_[j].val < 0) break;
      size_t home = mix64(slot_[j].key) & mask_;
      if (((j - home) & mask_) >= ((j - i) & mask_)) {
        slot_[i] = slot_[j];
        i = j;
      }
    }
    slot_[i].val = -1;
    --len_;
  }
  void reserve(size_t n) {
    if (8 * n > 5 * slot_.size()) rehash(n);
  }
  template <class F>
  void for_each(F f) const {
    for (const Slot& s : slot_)
      if (s.val >= 0) f(s.key, s.val);
  }

 private:
  struct Slot {
    uint64_t key;
    int64_t val;
  };
  void init(size_t n) {
    size_t c = 64;
    while (5 * c < 8 * n) c <<= 1;
    slot_.assign(c, Slot{0, -1});
    mask_ = c - 1;
    len_ = 0;
  }
  void put(uint64_t key, int64_t v) {
    size_t i = mix64(key) & mask_;
    while (slot_[i].val >= 0) i = (i + 1) & mask_;
    slot_[i] = Slot{key, v};
    ++len_;
  }
  void rehash(size_t n) {
    std::vector<Slot> old;
    old.swap(slot_);
    init(std::max(n, 2 * len_ + 2));
    for (const Slot& s : old)
      if (s.val >= 0) put(s.key, s.val);
  }
  std::vector<Slot> slot_;
  size_t mask_ = 0, len_ = 0;
};

// A registry split into kRegParts FlatTables by the top bits of its key's hash
// (the tables' slots use the low bits), so that host threads can check and
// insert the keys of different partitions at the same time.
constexpr int kRegParts = 16;
inline int reg_part(uint64_t key) { return (int)(mix64(key) >> 60); }

// Host worker threads for the parallel passes of bulk add_* calls.  Creating and joining 15 threads
// costs about a quarter of a millisecond, as much as one pass over a million items, and a bulk call
// makes four passes, so the workers stay and sleep on a condition variable between passes.  One pass
// runs at a time: a pass that finds the pool busy (a pass of another host thread, or one started from
// inside a pass, on a worker or on the calling thread) or that runs in a process forked after the pool
// started returns false, and the caller runs it on threads of its own.
class HostPool {
 public:
  static HostPool* get() {
    static std::mutex m;
    static HostPool* pool = nullptr;  // never destroyed: its workers sleep until the process ends
    std::lock_guard<std::mutex> g(m);
    if (!pool || pool->pid_ != getpid()) pool = new HostPool();
    return pool;
  }
  // f(t) for t = 0 .. T-1, t = 0 on the calling thread
  bool run(unsigned T, const std::function<void(unsigned)>& f) {
    if (in_pass_) return false;  // a pass inside a pass (the calling thread must not try busy_ twice)
    std::unique_lock<std::mutex> busy(busy_, std::try_to_lock);
    if (!busy.owns_lock() || T - 1 > workers_.size()) return false;
    in_pass_ = true;
    {
      std::lock_guard<std::mutex> g(m_);
      job_ = &f;
      job_threads_ = T;
      pending_ = T - 1;
      ++gen_;
    }
    work_.notify_all();
    f(0u);
    std::unique_lock<std::mutex> g(m_);
    done_.wait(g, [&] { return pending_ == 0; });
    job_ = nullptr;
    in_pass_ = false;
    return true;
  }

 private:
  HostPool() : pid_(getpid()) {
    const unsigned hw = std::thread::hardware_concurrency();
    const unsigned T = std::max(1u, std::min<unsigned>(hw ? hw : 1u, kRegParts));
    for (unsigned w = 1; w < T; ++w) {
      workers_.emplace_back([this, w] { loop(w); });
      workers_.back().detach();
    }
  }
  void loop(unsigned w) {
    in_pass_ = true;  // a worker runs nothing but passes
    uint64_t seen = 0;
    std::unique_lock<std::mutex> g(m_);
    for (;;) {
      work_.wait(g, [&] { return gen_ != seen; });
      seen = gen_;
      if (w >= job_threads_) continue;  // (a pass of fewer threads)
      const std::function<void(unsigned)>* job = job_;
      g.unlock();
      (*job)(w);
      g.lock();
      if (--pending_ == 0) done_.notify_one();
    }
  }
  const pid_t pid_;
  std::vector<std::thread> workers_;
  std::mutex busy_, m_;
  std::condition_variable work_, done_;
  const std::function<void(unsigned)>* job_ = nullptr;
  unsigned job_threads_ = 0, pending_ = 0;
  uint64_t gen_ = 0;
  static thread_local bool in_pass_;
};
thread_local bool HostPool::in_pass_ = false;

// f(t) on threads t = 0 .. T-1 (t = 0 on the calling thread): the pool's workers, else threads of its own
template <class F>
void run_threads(unsigned T, F f) {
  if (T > 1) {
    const std::function<void(unsigned)> job = [&f](unsigned t) { f(t); };
    if (HostPool::get()->run(T, job)) return;
  }
  std::vector<std::thread> th;
  for (unsigned t = 1; t < T; ++t) th.emplace_back(f, t);
  f(0u);
  for (auto& x : th) x.join();
}

// f(t, begin, end) over [0, n) in T contiguous chunks, chunk t on thread t
template <class F>
void parallel_chunks(unsigned T, size_t n, F f) {
  run_threads(T, [&](unsigned t) { f(t, n * t / T, n * (t + 1) / T); });
}

class PartTable {
 public:
  template <class Eq>
  int64_t find(uint64_t key, Eq eq) const {
    return part_[reg_part(key)].t.find(key, eq);
  }
  int64_t find(uint64_t key) const { return part_[reg_part(key)].t.find(key); }
  void prefetch(uint64_t key) const { part_[reg_part(key)].t.prefetch(key); }
  void insert(uint64_t key, int64_t v) { part_[reg_part(key)].t.insert(key, v); }
  void erase(uint64_t key, int64_t v) { part_[reg_part(key)].t.erase(key, v); }
  template <class F>
  void for_each(F f) const {
    for (const Part& p : part_) p.t.for_each(f);
  }
  // room for n entries spread over the partitions (a partition holds about n / kRegParts of them, within a
  // few percent for n in the thousands and up); large tables are set up by several threads
  void reserve(size_t n) {
    const size_t per = n / kRegParts + n / (32 * kRegParts) + 256;
    if (n < (size_t(1) << 16)) {
      for (Part& p : part_) p.t.reserve(per);
      return;
    }
    run_threads(kRegParts, [&](unsigned p) { part_[p].t.reserve(per); });
  }

 private:
  // one partition per cache-line pair: the threads inserting into different partitions never write
  // the same line (a table's entry count changes on every insert)
  struct alignas(128) Part {
    FlatTable t;
  };
  Part part_[kRegParts];
};

// Number -> index registry (node and element numbers, unique keys).  Numbers
// below a bound that follows the expected count (2 x reserved + 4096) live in
// a direct array, so the usual dense numbering costs no hashing and no cache
// miss per lookup; others fall back to a FlatTable.  A key stored in the table
// before the array grew over it is still found there.
class NumberMap {
 public:
  int64_t find(uint64_t key) const {
    if (key < dense_.size() && dense_[key] >= 0) return dense_[key];
    return table_.find(key);
  }
  void prefetch(uint64_t key) const {
    if (key < dense_.size()) __builtin_prefetch(&dense_[key]);
    else table_.prefetch(key);
  }
  void reserve(size_t total) {
    bound_ = std::max(bound_, 2 * total + 4096);
  }
  // Size the direct array for keys up to max_key before threads insert (inserts then never resize it).
  // Table entries whose keys the array now covers move into it, so a key below the array's size is
  // never in the table and each key has one home: its direct slot or its table partition.
  void fit(uint64_t max_key) {
    const size_t want = (size_t)std::min<uint64_t>(bound_, max_key + 1), have = dense_.size();
    if (want <= have) return;
    std::vector<std::pair<uint64_t, int64_t>> moved;
    table_.for_each([&](uint64_t k, int64_t v) {
      if (k < want) moved.emplace_back(k, v);
    });
    for (const auto& kv : moved) table_.erase(kv.first, kv.second);
    dense_.resize(want);  // no fill: the new slots are set to -1 by several threads
    const unsigned T = want - have >= (size_t(1) << 18) ? 8u : 1u;
    parallel_chunks(T, want - have, [&](unsigned, size_t b, size_t e) {
      std::fill(dense_.begin() + have + b, dense_.begin() + have + e, -1);
    });
    for (const auto& kv : moved) dense_[kv.first] = kv.second;
  }
  // the partition of a key for threaded inserts: blocks of 1024 direct slots (so that threads write
  // disjoint cache lines of the array), the table's hash partition beyond it
  int part(uint64_t key) const { return key < dense_.size() ? (int)((key >> 10) & (kRegParts - 1)) : reg_part(key); }
  void insert(uint64_t key, int64_t v) {
    if (key < bound_) {
      if (key >= dense_.size()) dense_.resize(std::min<size_t>(bound_, std::max<size_t>(key + 1, 2 * dense_.size())), -1);
      dense_[key] = v;
    } else {
      table_.insert(key, v);
    }
  }
  void erase(uint64_t key, int64_t v) {
    if (key < dense_.size() && dense_[key] == v) {
      dense_[key] = -1;
      return;
    }
    table_.erase(key, v);
  }

 private:
  HostVec<int64_t> dense_;
  PartTable table_;
  size_t bound_ = 4096;
};

uint64_t coord_hash(const CoordKey& k) { return mix64(k.a ^ mix64(k.b ^ mix64(k.c))); }
uint64_t set4_hash(const Set4& k) {
  return mix64(((uint64_t)k.s[0] << 32 | k.s[1]) ^ mix64((uint64_t)k.s[2] << 32 | k.s[3]));
}

unsigned grid_for(size_t n, unsigned block) { return (unsigned)((n + block - 1) / block); }

}  // namespace

// ---------------------------------------------------------------------------
// the handle
// ---------------------------------------------------------------------------
struct fem_gpu {
  double rel_tol = 0, abs_tol = 0;
  uint32_t nodes_number = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  // nodes
  size_t n_nodes = 0;
  HostVec<uint32_t> idx_number;
  HostVec<CoordKey> node_ck;  // normalised coordinate bits by index
  // node_coords holds the nodes [0, coords_built): bulk calls check coordinates on the GPU and leave the
  // host registry behind; a single-node call brings it up to date first
  size_t coords_built = 0;
  NumberMap node_idx;             // number -> index
  PartTable node_coords;          // coordinate hash -> index
  DevBuf<double> dx, dy, dz;
  DevBuf<double> stage;           // interleaved coordinates on their way in
  // elements
  std::vector<Run> runs;
  size_t n_pairs = 0;
  // truss
  size_t nt = 0;
  HostVec<uint32_t> t_num;
  NumberMap t_by_num;  // number -> element index
  PartTable t_pairs;   // node pair -> element index
  HostVec<uint32_t> t_nodes;  // node numbers per truss (2 each)
  size_t t_pairs_built = 0;       // t_pairs holds the trusses [0, t_pairs_built) (bulk calls check on the GPU)
  DevBuf<int32_t> t_n1, t_n2;
  DevBuf<double> t_E, t_A, t_A2;
  // beam
  size_t nbm = 0;
  HostVec<uint32_t> b_num;
  NumberMap b_by_num;
  PartTable b_pairs;
  HostVec<uint32_t> b_nodes;
  size_t b_pairs_built = 0;
  DevBuf<int32_t> b_n1, b_n2;
  DevBuf<double> b_E, b_nu, b_A, b_i11, b_i22, b_i12, b_it, b_ks, b_ax, b_ay, b_az;
  // plate
  size_t np = 0;
  HostVec<uint32_t> p_num, p_nodes;
  NumberMap p_by_num;
  PartTable p_sets;  // sorted node-number set hash -> element index
  size_t sets_built = 0;  // p_sets holds the plates [0, sets_built) (bulk calls check node sets on the GPU)
  DevBuf<int32_t> p_n1, p_n2, p_n3, p_n4;
  DevBuf<double> p_E, p_nu, p_t, p_ks;
  // loads: nodal contributions (DOF, value) in call order and the forces vector they sum to
  DevBuf<unsigned long long> ld_key;
  DevBuf<double> ld_val, forces;
  size_t n_ld = 0;
  bool forces_valid = false;
  // sparse separation (K_aa, K_ab, K_ba, K_bb)
  bool sep_valid = false;
  DevBuf<uint8_t> sep_imposed, sep_cls;
  DevBuf<uint32_t> sep_u32;             // class flags, local positions, per-row counts
  DevBuf<unsigned long long> sep_scan;  // per block: row starts by global row (n + 1 each)
  DevBuf<unsigned long long> sep_err;
  DevBuf<int64_t> sep_idx;              // a list, then b list
  DevBuf<int64_t> sep_rp[4];
  DevBuf<int32_t> sep_ci[4];
  DevBuf<double> sep_v[4];
  int64_t sep_n[2] = {0, 0}, sep_nnz[4] = {0, 0, 0, 0};
  // PCG on K_aa: vectors, dot-product partials, preconditioner blocks and their inverses
  DevBuf<double> pcg_vec, pcg_part, pcg_scal, pcg_inv;
  DevBuf<uint32_t> pcg_blk, pcg_info;
  DevBuf<int> pcg_state;
  // sliced ELLPACK copy of K_aa for the PCG's products (valid with the separation it was built from)
  bool sell_valid = false;
  size_t sell_windows = 0;
  int64_t sell_entries = 0;
  DevBuf<int64_t> sell_off;
  DevBuf<uint32_t> sell_perm;
  DevBuf<int32_t> sell_col;
  DevBuf<double> sell_val;
  // validation scratch
  DevBuf<int> vstatus;
  DevBuf<unsigned long long> vfirst;
  // symbolic results
  bool pattern_valid = false;
  size_t n_blocks = 0;
  DevBuf<uint32_t> slot_t, slot_b, slot_p;
  DevBuf<uint64_t> mask_t, mask_b, mask_p;
  DevBuf<unsigned long long> off_t, off_b, off_p, blk_voff;  // packed offsets (offset | packing << 62)
  DevBuf<uint8_t> blk_lay;
  DevBuf<uint64_t> blk_pmask;  // pattern bits over packed positions
  DevBuf<unsigned long long> sbase;  // kSlotCats x (n_blocks + 1) slot scans
  unsigned long long slot_off[kSlotCats] = {0, 0, 0, 0, 0};
  unsigned long long vs_off = 0;     // S starts here in V
  size_t n_desc = 0;
  DevBuf<uint32_t> src_map;          // per CSR entry: its slot in S
  DevBuf<uint2> slot_desc;           // per slot: scratch start, count | stride << 24 | in-pattern << 31
  size_t s_words = 0;
  size_t v_words = 0;
  size_t v_pad = 0;    // of which padding words (never read: one per contribution of a 13-entry block)
  DevBuf<double> V;
  DevBuf<uint32_t> blk_start, blk_count;
  DevBuf<uint64_t> blk_mask, blk_maskT;
  DevBuf<int32_t> blk_I, blk_J;
  DevBuf<int64_t> row_ptr;
  DevBuf<int32_t> col_idx;
  DevBuf<double> values;
  int64_t nnz = 0, n_groups = 0;
  DevBuf<int32_t> g_row, g_col, nnz_group;
  DevBuf<uint8_t> g_kind;
  DevBuf<int> flag;
  DevBuf<uint8_t> cub_tmp;
  bool numeric_done = false;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  float t_elem_ms = 0, t_reduce_ms = 0;
  // the numeric pass as a CUDA graph (captured at its first launch after each symbolic phase)
  cudaGraphExec_t num_graph = nullptr;
  // a second stream for pattern read-backs that overlap the numeric pass (fem_gpu_assemble_to_host)
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t copy_ev = nullptr;
  cudaEvent_t fill_ev[4] = {};  // the row fill's node chunks done (their columns can go back)
  bool num_eager_done = false;  // the first numeric pass since the graph was dropped has run (uncaptured)
  void drop_numeric_graph() {
    if (num_graph) cudaGraphExecDestroy(num_graph);
    num_graph = nullptr;
    num_eager_done = false;
  }
  // vector-Jacobian product
  bool vjp_inc_valid = false;
  DevBuf<int64_t> vjp_inc_off, vjp_inc;
  DevBuf<double> vjp_in, vjp_uT, vjp_lT, vjp_Ws, vjp_gc, vjp_gp, vjp_gxyz;
  DevBuf<uint32_t> vjp_pblk;  // stiffness block of every element node pair
  float t_vjp_ms = 0;
  // element results: staged displacements and results, and the events around the result kernels
  DevBuf<double> res_buf;
  cudaEvent_t res_ev[2] = {nullptr, nullptr};
  bool res_timed = false;

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
  NodesView nodes() const { return NodesView{dx.p, dy.p, dz.p, dx.cap}; }
  BeamView beams() const {
    return BeamView{b_n1.p, b_n2.p, b_E.p, b_nu.p, b_A.p, b_i11.p, b_i22.p, b_i12.p, b_it.p, b_ks.p, b_ax.p, b_ay.p, b_az.p};
  }
  PlateView plates() const { return PlateView{p_n1.p, p_n2.p, p_n3.p, p_n4.p, p_E.p, p_nu.p, p_t.p, p_ks.p}; }
  TrussView trusses() const { return TrussView{t_n1.p, t_n2.p, t_E.p, t_A.p, t_A2.p}; }
  void append_run(int kind, size_t begin, size_t count) {
    if (!count) return;
    size_t ppe = kind == kPlate ? kPairs4 : kPairs2;
    runs.push_back(Run{kind, begin, count, n_pairs});
    n_pairs += count * ppe;
    pattern_valid = false;
    vjp_inc_valid = false;
    numeric_done = false;
    drop_numeric_graph();
  }
};

#define CK(call)                                         \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return h->cuda_fail(e_, #call); \
  } while (0)

namespace {

template <class T>
cudaError_t upload(DevBuf<T>& buf, size_t at, const T* src, size_t n, cudaStream_t s) {
  cudaError_t e = buf.reserve(at + n, s, at);
  if (e != cudaSuccess) return e;
  if (!n) return cudaSuccess;
  return cudaMemcpyAsync(buf.p + at, src, n * sizeof(T), cudaMemcpyHostToDevice, s);
}

// runs the validation kernel over [begin, begin+count) and returns the first
// failing offset (or count) and its status code
// ---- duplicate checks of bulk calls on the GPU ------------------------------------------------------------
// Items are grouped by a 63-bit hash of their key (radix sort of (hash, item), stable, so a group lists its
// items in call order); inside a group an item is compared exactly with the earlier ones.  The result is the
// smallest item equal to an earlier item -- the first failure a sequential pass over the registry would meet.
__device__ __forceinline__ unsigned long long dev_mix64(unsigned long long x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ull;
  x ^= x >> 33;
  return x;
}
constexpr unsigned long long kNoKey = ~0ull;  // items that equal nothing sort last

// node coordinates: the model's nodes [0, start) on the device (SoA), then the call's nodes (interleaved)
struct CoordSource {
  const double *x, *y, *z, *xyz;
  size_t start;
  __device__ __forceinline__ void get(size_t i, double& a, double& b, double& c) const {
    if (i < start) {
      a = x[i];
      b = y[i];
      c = z[i];
    } else {
      const double* p = xyz + 3 * (i - start);
      a = p[0];
      b = p[1];
      c = p[2];
    }
  }
};

__global__ void k_coord_keys(size_t n, CoordSource src, unsigned long long* __restrict__ key, uint32_t* __restrict__ idx) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double a, b, c;
  src.get(i, a, b, c);
  idx[i] = (uint32_t)i;
  if (a != a || b != b || c != c) {  // NaN coordinates equal no other (the reference compares with ==)
    key[i] = kNoKey;
    return;
  }
  if (a == 0.0) a = 0.0;  // -0.0 == 0.0
  if (b == 0.0) b = 0.0;
  if (c == 0.0) c = 0.0;
  const unsigned long long ha = (unsigned long long)__double_as_longlong(a),
                           hb = (unsigned long long)__double_as_longlong(b),
                           hc = (unsigned long long)__double_as_longlong(c);
  key[i] = dev_mix64(ha ^ dev_mix64(hb ^ dev_mix64(hc))) >> 1;
}

__global__ void k_coord_dups(size_t n, const unsigned long long* __restrict__ skey, const uint32_t* __restrict__ sidx,
                             CoordSource src, unsigned long long* first) {
  const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k == 0 || k >= n || skey[k] == kNoKey || skey[k - 1] != skey[k]) return;
  const uint32_t j = sidx[k];
  double a, b, c;
  src.get(j, a, b, c);
  for (size_t p = k; p-- > 0 && skey[p] == skey[k];) {
    double a2, b2, c2;
    src.get(sidx[p], a2, b2, c2);
    if (a2 == a && b2 == b && c2 == c) {
      atomicMin(first, (unsigned long long)j);
      return;
    }
  }
}

// plate node sets (node indexes, which map one to one to node numbers), sorted by a comparator network
__device__ __forceinline__ uint4 dev_sorted4(int32_t p, int32_t q, int32_t r, int32_t s) {
  uint32_t a = (uint32_t)p, b = (uint32_t)q, c = (uint32_t)r, d = (uint32_t)s, t;
#define FEM_DSWAP(x, y) \
  if (y < x) {          \
    t = x;              \
    x = y;              \
    y = t;              \
  }
  FEM_DSWAP(a, b)
  FEM_DSWAP(c, d)
  FEM_DSWAP(a, c)
  FEM_DSWAP(b, d)
  FEM_DSWAP(b, c)
#undef FEM_DSWAP
  return make_uint4(a, b, c, d);
}

__global__ void k_set4_keys(size_t n, const int32_t* __restrict__ n1, const int32_t* __restrict__ n2,
                            const int32_t* __restrict__ n3, const int32_t* __restrict__ n4,
                            unsigned long long* __restrict__ key, uint32_t* __restrict__ idx) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint4 v = dev_sorted4(n1[i], n2[i], n3[i], n4[i]);
  idx[i] = (uint32_t)i;
  key[i] = dev_mix64(((unsigned long long)v.x << 32 | v.y) ^ dev_mix64((unsigned long long)v.z << 32 | v.w)) >> 1;
}

__global__ void k_set4_dups(size_t n, const unsigned long long* __restrict__ skey, const uint32_t* __restrict__ sidx,
                            const int32_t* __restrict__ n1, const int32_t* __restrict__ n2,
                            const int32_t* __restrict__ n3, const int32_t* __restrict__ n4, unsigned long long* first) {
  const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k == 0 || k >= n || skey[k - 1] != skey[k]) return;
  const uint32_t j = sidx[k];
  const uint4 v = dev_sorted4(n1[j], n2[j], n3[j], n4[j]);
  for (size_t p = k; p-- > 0 && skey[p] == skey[k];) {
    const uint32_t i = sidx[p];
    const uint4 w = dev_sorted4(n1[i], n2[i], n3[i], n4[i]);
    if (w.x == v.x && w.y == v.y && w.z == v.z && w.w == v.w) {
      atomicMin(first, (unsigned long long)j);
      return;
    }
  }
}

// a cub device-wide call: size query, temporary storage from the handle, the call
template <class F>
int cub_call(fem_gpu* h, F f) {
  size_t bytes = 0;
  CK(f((void*)nullptr, bytes));
  CK(h->cub_tmp.reserve(bytes ? bytes : 1, h->stream));
  CK(f((void*)h->cub_tmp.p, bytes));
  return FEM_GPU_OK;
}

// The smallest of the items [0, total) that equals an earlier item (total when none), in two steps so
// that host work runs while the GPU searches: dup_start enqueues the key kernel keys(key, idx) over
// [0, total), a stable radix sort of (key, item) and the comparison dups(skey, sidx, first) over the
// sorted items; dup_finish waits for the result.
struct DupSearch {
  DevBuf<unsigned long long> key, skey, out;
  DevBuf<uint32_t> idx, sidx;
  size_t total = 0;
};

template <class Keys, class Dups>
int dup_start(fem_gpu* h, DupSearch& d, size_t total, Keys keys, Dups dups) {
  d.total = total;
  if (total < 2) return FEM_GPU_OK;
  cudaStream_t s = h->stream;
  CK(d.key.reserve(total, s));
  CK(d.skey.reserve(total, s));
  CK(d.idx.reserve(total, s));
  CK(d.sidx.reserve(total, s));
  CK(d.out.reserve(1, s));
  const unsigned long long none = total;
  CK(cudaMemcpyAsync(d.out.p, &none, sizeof none, cudaMemcpyHostToDevice, s));
  keys(d.key.p, d.idx.p);
  CK(cudaGetLastError());
  int st = cub_call(h, [&](void* tmp, size_t& bytes) {
    return cub::DeviceRadixSort::SortPairs(tmp, bytes, d.key.p, d.skey.p, d.idx.p, d.sidx.p, (int64_t)total, 0, 64, s);
  });
  if (st) return st;
  dups(d.skey.p, d.sidx.p, d.out.p);
  CK(cudaGetLastError());
  return FEM_GPU_OK;
}

int dup_finish(fem_gpu* h, DupSearch& d, size_t* first) {
  *first = d.total;
  if (d.total < 2) return FEM_GPU_OK;
  unsigned long long f = 0;
  CK(cudaMemcpyAsync(&f, d.out.p, sizeof f, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  *first = (size_t)f;
  return FEM_GPU_OK;
}

// two-node elements: the node pair itself (smaller index high) is the key, so equal keys are equal pairs
__global__ void k_pair_keys(size_t n, const int32_t* __restrict__ n1, const int32_t* __restrict__ n2,
                            unsigned long long* __restrict__ key, uint32_t* __restrict__ idx) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t a = (uint32_t)n1[i], b = (uint32_t)n2[i];
  key[i] = a < b ? ((unsigned long long)a << 32 | b) : ((unsigned long long)b << 32 | a);
  idx[i] = (uint32_t)i;
}

__global__ void k_pair_dups(size_t n, const unsigned long long* __restrict__ skey, const uint32_t* __restrict__ sidx,
                            unsigned long long* first) {
  const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k == 0 || k >= n || skey[k - 1] != skey[k]) return;
  atomicMin(first, (unsigned long long)sidx[k]);
}

// The first of the items [0, count) that the validation kernel launch(status, first) rejects, with its error code
// (*first_bad = count when none).  validate_start enqueues the kernel over `launched` items; validate_finish
// waits and reports the first rejected item below `count` (<= launched): a bulk call can start the kernel
// before its host checks have settled how many items get that far.
template <class Launch>
int validate_start(fem_gpu* h, size_t launched, Launch launch) {
  if (!launched) return FEM_GPU_OK;
  CK(h->vstatus.reserve(launched, h->stream));
  CK(h->vfirst.reserve(1, h->stream));
  unsigned long long init = ~0ull;
  CK(cudaMemcpyAsync(h->vfirst.p, &init, sizeof init, cudaMemcpyHostToDevice, h->stream));
  launch(h->vstatus.p, h->vfirst.p);
  CK(cudaGetLastError());
  return FEM_GPU_OK;
}
int validate_finish(fem_gpu* h, size_t count, size_t* first_bad, int* code) {
  *first_bad = count;
  *code = 0;
  if (!count) return FEM_GPU_OK;
  unsigned long long first = 0;
  CK(cudaMemcpyAsync(&first, h->vfirst.p, sizeof first, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (first != ~0ull && first < count) {
    int c = 0;
    CK(cudaMemcpy(&c, h->vstatus.p + first, sizeof c, cudaMemcpyDeviceToHost));
    *first_bad = (size_t)first;
    *code = c;
  }
  return FEM_GPU_OK;
}
template <class Launch, class Host>
int first_failure(fem_gpu* h, size_t count, Launch launch, Host host, size_t* first_bad, int* code) {
  *first_bad = count;
  *code = 0;
  if (!count) return FEM_GPU_OK;
  int st = validate_start(h, count, launch);
  if (st) return st;
  host();  // host work that does not wait for the result runs while the GPU validates
  return validate_finish(h, count, first_bad, code);
}

int ensure_ready(fem_gpu* h) {
  if (!h) return FEM_GPU_ERR_ARGUMENT;
  if (h->stream) return FEM_GPU_OK;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return h->cuda_fail(e, "cudaGetDevice");
  CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  for (auto& ev : h->ev) CK(cudaEventCreate(&ev));
  size_t nn = h->nodes_number ? h->nodes_number : 1;
  CK(h->dx.reserve(nn, h->stream));
  CK(h->dy.reserve(nn, h->stream));
  CK(h->dz.reserve(nn, h->stream));
  CK(h->flag.reserve(2, h->stream));  // [0] numeric pass, [1] symbolic phase
  return FEM_GPU_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" int fem_gpu_create(double rel_tol, double abs_tol, uint32_t nodes_number, fem_gpu_t** out) {
  if (!out) return FEM_GPU_ERR_ARGUMENT;
  fem_gpu* h = new fem_gpu();
  h->rel_tol = rel_tol;
  h->abs_tol = abs_tol;
  h->nodes_number = nodes_number;
  h->idx_number.reserve(nodes_number);
  *out = h;
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_release_cached_memory(void) {
  cudaMemPool_t pool = nullptr;
  cudaError_t e = device_pool(&pool);
  if (e != cudaSuccess) return FEM_GPU_ERR_CUDA;
  e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return FEM_GPU_ERR_CUDA;
  return cudaMemPoolTrimTo(pool, 0) == cudaSuccess ? FEM_GPU_OK : FEM_GPU_ERR_CUDA;
}

extern "C" int fem_gpu_destroy(fem_gpu_t* h) {
  if (!h) return FEM_GPU_OK;
  // work of any stream may still read the model's arrays (device pointers handed out): wait for all of it
  // before the arrays go back to the pool
  cudaDeviceSynchronize();
  DevBuf<double>* d[] = {&h->dx, &h->dy, &h->dz, &h->stage, &h->t_E, &h->t_A, &h->t_A2, &h->b_E, &h->b_nu, &h->b_A,
                         &h->b_i11, &h->b_i22, &h->b_i12, &h->b_it, &h->b_ks, &h->b_ax, &h->b_ay, &h->b_az,
                         &h->p_E, &h->p_nu, &h->p_t, &h->p_ks, &h->V, &h->values};
  for (auto* b : d) b->release();
  DevBuf<int32_t>* i[] = {&h->t_n1, &h->t_n2, &h->b_n1, &h->b_n2, &h->p_n1, &h->p_n2, &h->p_n3, &h->p_n4,
                          &h->blk_I, &h->blk_J, &h->col_idx, &h->g_row, &h->g_col, &h->nnz_group};
  for (auto* b : i) b->release();
  h->slot_t.release();
  h->slot_b.release();
  h->slot_p.release();
  h->off_t.release();
  h->off_b.release();
  h->off_p.release();
  h->blk_voff.release();
  h->blk_lay.release();
  h->blk_pmask.release();
  h->sbase.release();
  h->src_map.release();
  h->slot_desc.release();
  h->mask_t.release();
  h->mask_b.release();
  h->mask_p.release();
  h->blk_start.release();
  h->blk_count.release();
  h->blk_mask.release();
  h->blk_maskT.release();
  h->row_ptr.release();
  h->g_kind.release();
  h->flag.release();
  h->cub_tmp.release();
  h->vjp_pblk.release();
  for (DevBuf<double>* v : {&h->vjp_in, &h->vjp_uT, &h->vjp_lT, &h->vjp_Ws, &h->vjp_gc, &h->vjp_gp, &h->vjp_gxyz})
    v->release();
  h->vjp_inc_off.release();
  h->vjp_inc.release();
  h->vstatus.release();
  h->vfirst.release();
  h->ld_key.release();
  h->ld_val.release();
  h->forces.release();
  for (DevBuf<double>* v : {&h->pcg_vec, &h->pcg_part, &h->pcg_scal, &h->pcg_inv}) v->release();
  h->pcg_blk.release();
  h->pcg_info.release();
  h->pcg_state.release();
  h->sell_off.release();
  h->sell_perm.release();
  h->sell_col.release();
  h->sell_val.release();
  h->sep_imposed.release();
  h->sep_cls.release();
  h->sep_u32.release();
  h->sep_scan.release();
  h->sep_err.release();
  h->sep_idx.release();
  for (int b = 0; b < 4; ++b) {
    h->sep_rp[b].release();
    h->sep_ci[b].release();
    h->sep_v[b].release();
  }
  h->res_buf.release();
  h->drop_numeric_graph();
  if (h->copy_ev) cudaEventDestroy(h->copy_ev);
  for (auto& ev : h->fill_ev)
    if (ev) cudaEventDestroy(ev);
  if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
  for (auto& ev : h->ev)
    if (ev) cudaEventDestroy(ev);
  for (auto& ev : h->res_ev)
    if (ev) cudaEventDestroy(ev);
  // the remaining device arrays are freed by their destructors, in the stream's order: the stream goes last
  cudaStream_t s = h->stream;
  delete h;
  if (s) cudaStreamDestroy(s);
  return FEM_GPU_OK;
}

extern "C" const char* fem_gpu_last_error(const fem_gpu_t* h) { return h ? h->err.c_str() : "null handle"; }

namespace {
// Bulk add_* calls of at least this many items check their registries on several host threads.
constexpr size_t kParallelAdd = size_t(1) << 15;

unsigned add_threads() {
  const unsigned hw = std::thread::hardware_concurrency();
  return std::max(1u, std::min<unsigned>(hw ? hw : 1u, kRegParts));
}

// dst += src[0, count), by several threads for bulk calls (a fresh array's first touch is most of the cost)
void append_host(HostVec<uint32_t>& dst, const uint32_t* src, size_t count) {
  const size_t at = dst.size();
  dst.resize(at + count);
  if (count < kParallelAdd) {
    if (count) std::memcpy(dst.data() + at, src, count * sizeof(uint32_t));
    return;
  }
  parallel_chunks(add_threads(), count, [&](unsigned, size_t b, size_t e) {
    std::memcpy(dst.data() + at + b, src + b, (e - b) * sizeof(uint32_t));
  });
}

// the thread (of T) that owns a registry partition; 0xff for an item without a key
struct PartOwner {
  uint8_t of[kRegParts];
  explicit PartOwner(unsigned T) {
    for (int p = 0; p < kRegParts; ++p) of[p] = (uint8_t)(p % T);
  }
  uint8_t operator()(uint64_t key) const { return of[reg_part(key)]; }
  uint8_t of_part(int p) const { return of[p]; }
};

// The duplicate checks of a bulk add, in call order, on T host threads.  Item k has up to two
// registry keys (roles A and B); own_a[k], own_b[k] are the threads owning their partitions (0xff:
// no key).  The owner checks and inserts its partitions' keys in item order -- fa(k) / fb(k) return
// false on a duplicate, else insert -- so every check sees the entries of exactly the earlier items
// and calls, as one sequential pass would.  A thread stops at its first duplicate; the first failing
// item is the smallest of those (role A before role B on the same item), items from `limit` on are
// not looked at.  Returns that item (or limit) and sets *role to 1 (A), 2 (B) or 0.
// pa(k) / pb(k) prefetch the registry slots of item k's keys, issued a few of the thread's own items ahead.
template <class FA, class FB, class PA, class PB>
size_t registry_pass(unsigned T, size_t limit, const uint8_t* own_a, const uint8_t* own_b, FA fa, FB fb, PA pa,
                     PB pb, int* role) {
  std::vector<size_t> first(T, limit);
  std::vector<int> which(T, 0);
  // every thread's checks as a list in item order (k << 1 | role B), made by a counting pass over T chunks, so
  // that a thread walks its own items only rather than all of them
  std::vector<size_t> cnt((size_t)T * T, 0), at((size_t)T * T, 0), len(T, 0);
  parallel_chunks(T, limit, [&](unsigned c, size_t b, size_t e) {
    size_t* n = &cnt[(size_t)c * T];
    for (size_t k = b; k < e; ++k) {
      if (own_a[k] < T) ++n[own_a[k]];
      if (own_b[k] < T) ++n[own_b[k]];
    }
  });
  for (unsigned t = 0; t < T; ++t) {
    size_t run = 0;
    for (unsigned c = 0; c < T; ++c) {
      at[(size_t)c * T + t] = run;
      run += cnt[(size_t)c * T + t];
    }
    len[t] = run;
  }
  std::vector<HostVec<uint64_t>> list(T);
  run_threads(T, [&](unsigned t) { list[t].resize(len[t]); });
  parallel_chunks(T, limit, [&](unsigned c, size_t b, size_t e) {
    size_t* pos = &at[(size_t)c * T];
    for (size_t k = b; k < e; ++k) {
      if (own_a[k] < T) list[own_a[k]][pos[own_a[k]]++] = (uint64_t)k << 1;
      if (own_b[k] < T) list[own_b[k]][pos[own_b[k]]++] = ((uint64_t)k << 1) | 1u;
    }
  });
  run_threads(T, [&](unsigned t) {
    const HostVec<uint64_t>& my = list[t];
    const size_t m = my.size(), ahead = 8;
    for (size_t q = 0; q < m; ++q) {
      if (q + ahead < m) {
        const uint64_t w = my[q + ahead];
        if (w & 1u) pb((size_t)(w >> 1));
        else pa((size_t)(w >> 1));
      }
      const uint64_t w = my[q];
      const size_t k = (size_t)(w >> 1);
      if (!(w & 1u) ? !fa(k) : !fb(k)) {
        first[t] = k;
        which[t] = (w & 1u) ? 2 : 1;
        return;
      }
    }
  });
  size_t f = limit;
  *role = 0;
  for (unsigned t = 0; t < T; ++t)
    if (first[t] < f || (first[t] == f && which[t] && (*role == 0 || which[t] < *role))) {
      f = first[t];
      *role = which[t];
    }
  return f;
}
}  // namespace

namespace {
// Registry entries of items that bulk calls checked on the GPU go in when a call first needs the host
// registry: keys in parallel, then each thread inserts its partitions' keys in item order.
template <class Key>
void registry_catch_up(PartTable& reg, size_t b0, size_t n, Key key) {
  if (!n) return;
  const unsigned T = n >= kParallelAdd ? add_threads() : 1u;
  const PartOwner owner(T);
  HostVec<uint64_t> hs(n);
  HostVec<uint8_t> own(n);
  parallel_chunks(T, n, [&](unsigned, size_t b, size_t e) {
    for (size_t q = b; q < e; ++q) {
      uint64_t k = 0;
      own[q] = key(b0 + q, &k) ? owner(k) : (uint8_t)0xff;
      hs[q] = k;
    }
  });
  run_threads(T, [&](unsigned t) {
    const size_t ahead = 8 * (size_t)T;
    for (size_t q = 0; q < n; ++q) {
      if (q + ahead < n && own[q + ahead] == t) reg.prefetch(hs[q + ahead]);
      if (own[q] == t) reg.insert(hs[q], (int64_t)(b0 + q));
    }
  });
}

void ensure_coords(fem_gpu* h) {
  if (h->coords_built >= h->n_nodes) return;
  h->node_coords.reserve(h->n_nodes);
  registry_catch_up(h->node_coords, h->coords_built, h->n_nodes - h->coords_built, [&](size_t i, uint64_t* k) {
    const CoordKey& ck = h->node_ck[i];
    double x, y, z;
    memcpy(&x, &ck.a, 8);
    memcpy(&y, &ck.b, 8);
    memcpy(&z, &ck.c, 8);
    if (!(x == x && y == y && z == z)) return false;  // NaN coordinates are never equal to any
    *k = coord_hash(ck);
    return true;
  });
  h->coords_built = h->n_nodes;
}

void ensure_pairs(PartTable& reg, size_t* built, size_t count, const HostVec<uint32_t>& nodes) {
  if (*built >= count) return;
  reg.reserve(count);
  registry_catch_up(reg, *built, count - *built, [&](size_t e, uint64_t* k) {
    *k = pair_key(nodes[2 * e], nodes[2 * e + 1]);
    return true;
  });
  *built = count;
}

void ensure_sets(fem_gpu* h) {
  if (h->sets_built >= h->np) return;
  h->p_sets.reserve(h->np);
  registry_catch_up(h->p_sets, h->sets_built, h->np - h->sets_built, [&](size_t e, uint64_t* k) {
    *k = set4_hash(sorted4(&h->p_nodes[4 * e]));
    return true;
  });
  h->sets_built = h->np;
}
}  // namespace

// add_node, methods_for_node_data_handle.rs:39-79
extern "C" int fem_gpu_add_nodes(fem_gpu_t* h, const uint32_t* numbers, const double* xyz, size_t n,
                                 size_t* n_added) {
  if (n_added) *n_added = 0;
  if (!h || (n && (!numbers || !xyz))) return FEM_GPU_ERR_ARGUMENT;
  int st = ensure_ready(h);
  if (st) return st;
  h->drop_numeric_graph();  // the element and node arrays may move
  size_t start = h->n_nodes, k = 0;
  int code = FEM_GPU_OK;
  h->node_idx.reserve(h->n_nodes + n);
  h->node_ck.reserve(h->n_nodes + n);
  h->idx_number.reserve(h->n_nodes + n);
  if (n >= kParallelAdd) {
    // keys of every node, then the registry pass on host threads (same checks, same first failure)
    const unsigned T = add_threads();
    const size_t room = h->nodes_number > start ? (size_t)h->nodes_number - start : 0;
    const size_t limit = std::min(n, room);
    const PartOwner owner(T);
    HostVec<uint8_t> pa(n), pb(n, 0xff);  // role B (coordinates) is checked on the GPU
    std::vector<uint32_t> tmax(T, 0);
    h->node_ck.resize(start + n);
    h->idx_number.resize(start + n);
    // the call's coordinates go up first: the GPU looks for the smallest new node equal to an earlier node (of
    // the model or of the call) while the host checks the numbers
    CK(upload(h->stage, 0, xyz, 3 * n, h->stream));
    const CoordSource src{h->dx.p, h->dy.p, h->dz.p, h->stage.p, start};
    const size_t total = start + n;
    DupSearch dup;
    st = dup_start(
        h, dup, total,
        [&](unsigned long long* key, uint32_t* idx) {
          k_coord_keys<<<grid_for(total, 256), 256, 0, h->stream>>>(total, src, key, idx);
        },
        [&](const unsigned long long* skey, const uint32_t* sidx, unsigned long long* out) {
          k_coord_dups<<<grid_for(total, 256), 256, 0, h->stream>>>(total, skey, sidx, src, out);
        });
    if (st) return st;
    parallel_chunks(T, n, [&](unsigned t, size_t b, size_t e) {
      uint32_t mx = 0;
      for (size_t q = b; q < e; ++q) {
        h->node_ck[start + q] = coord_key(xyz[3 * q], xyz[3 * q + 1], xyz[3 * q + 2]);
        h->idx_number[start + q] = numbers[q];
        mx = std::max(mx, numbers[q]);
      }
      tmax[t] = mx;
    });
    h->node_idx.fit(*std::max_element(tmax.begin(), tmax.end()));
    parallel_chunks(T, n, [&](unsigned, size_t b, size_t e) {
      for (size_t q = b; q < e; ++q) pa[q] = owner.of_part(h->node_idx.part(numbers[q]));
    });
    int role = 0;
    size_t f = registry_pass(
        T, limit, pa.data(), pb.data(),
        [&](size_t q) {
          if (h->node_idx.find(numbers[q]) >= 0) return false;
          h->node_idx.insert(numbers[q], (int64_t)(start + q));
          return true;
        },
        [&](size_t) { return true; }, [&](size_t q) { h->node_idx.prefetch(numbers[q]); }, [&](size_t) {}, &role);
    size_t fc = total;
    st = dup_finish(h, dup, &fc);
    if (st) return st;
    if (fc >= start && fc - start < f) {  // (nodes of the model are distinct: fc < start cannot happen)
      f = fc - start;
      role = 2;
    }
    for (size_t q = f; q < limit; ++q)  // entries of items at or after the first failure go again
      h->node_idx.erase(numbers[q], (int64_t)(start + q));
    h->node_ck.resize(start + f);
    h->idx_number.resize(start + f);
    h->n_nodes = start + f;
    k = f;
    if (f < n) {
      if (role == 1) {
        code = h->fail(FEM_GPU_ERR_NODE_NUMBER, "Node with number %u already exists!", numbers[f]);
      } else if (role == 2) {
        code = h->fail(FEM_GPU_ERR_NODE_COORDS, "Node with coordinates x: %s, y: %s, z: %s already exists!",
                       rust_f64(xyz[3 * f]).c_str(), rust_f64(xyz[3 * f + 1]).c_str(),
                       rust_f64(xyz[3 * f + 2]).c_str());
      } else {
        code = h->fail(FEM_GPU_ERR_NODE_LIMIT, "Nodes number could not be greater than %u!", h->nodes_number);
      }
    }
  }
  constexpr size_t kAhead = 8;  // prefetch distance (entries) into the coordinate registry
  if (n < kParallelAdd) {
    ensure_coords(h);
    h->node_coords.reserve(h->n_nodes + n);
  }
  if (n < kParallelAdd)
    for (size_t q = 0; q < std::min(n, kAhead); ++q)
      h->node_coords.prefetch(coord_hash(coord_key(xyz[3 * q], xyz[3 * q + 1], xyz[3 * q + 2])));
  for (; k < n && n < kParallelAdd; ++k) {
    if (k + kAhead < n) {
      const double* f = xyz + 3 * (k + kAhead);
      h->node_coords.prefetch(coord_hash(coord_key(f[0], f[1], f[2])));
      h->node_idx.prefetch(numbers[k + kAhead]);
    }
    uint32_t num = numbers[k];
    double x = xyz[3 * k], y = xyz[3 * k + 1], z = xyz[3 * k + 2];
    size_t index = h->n_nodes;
    if (h->nodes_number == 0 || index > (size_t)h->nodes_number - 1) {
      code = h->fail(FEM_GPU_ERR_NODE_LIMIT, "Nodes number could not be greater than %u!", h->nodes_number);
      break;
    }
    if (h->node_idx.find(num) >= 0) {
      code = h->fail(FEM_GPU_ERR_NODE_NUMBER, "Node with number %u already exists!", num);
      break;
    }
    CoordKey ck = coord_key(x, y, z);
    if (x == x && y == y && z == z) {
      uint64_t hk = coord_hash(ck);
      const HostVec<CoordKey>& known = h->node_ck;
      if (h->node_coords.find(hk, [&](int64_t i) { return known[(size_t)i] == ck; }) >= 0) {
        code = h->fail(FEM_GPU_ERR_NODE_COORDS, "Node with coordinates x: %s, y: %s, z: %s already exists!",
                       rust_f64(x).c_str(), rust_f64(y).c_str(), rust_f64(z).c_str());
        break;
      }
      h->node_coords.insert(hk, (int64_t)index);
    }
    h->node_idx.insert(num, (int64_t)index);
    h->node_ck.push_back(ck);
    h->idx_number.push_back(num);
    h->n_nodes++;
  }
  if (n < kParallelAdd) h->coords_built = h->n_nodes;
  if (n_added) *n_added = k;
  size_t m = h->n_nodes - start;
  if (m) {
    // the accepted prefix of the caller's interleaved xyz goes up as is (bulk calls sent it already) and is
    // split on the device
    if (n < kParallelAdd) CK(upload(h->stage, 0, xyz, 3 * m, h->stream));
    k_split_xyz<<<grid_for(m, 256), 256, 0, h->stream>>>(m, h->stage.p, h->dx.p + start, h->dy.p + start,
                                                         h->dz.p + start);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->stream));
    h->pattern_valid = false;
    h->numeric_done = false;
  }
  return code;
}

namespace {
constexpr size_t kRegAhead = 8;  // prefetch distance (elements) into the registries of the bulk add_* loops


int lookup_node(fem_gpu* h, uint32_t num, int32_t* idx) {
  int64_t i = h->node_idx.find(num);
  if (i < 0) return h->fail(FEM_GPU_ERR_NODE_NOT_EXIST, "Node with number %u does not exist!", num);
  *idx = (int32_t)i;
  return FEM_GPU_OK;
}

// The host checks of a bulk add of two-node elements (trusses, beams) on host threads, in the
// sequential loop's order: both nodes exist, the number is new, the node pair is new.  Returns the
// status of the first failing item (message set as the sequential loop would set it); *passed is
// the number of items before it, whose node indices are in i1, i2.
int two_node_checks(fem_gpu* h, const char* kind, NumberMap& by_num, DevBuf<int32_t>& dn1, DevBuf<int32_t>& dn2,
                    size_t base, const uint32_t* numbers, const uint32_t* nodes, size_t n, HostVec<int32_t>& i1,
                    HostVec<int32_t>& i2, size_t* passed) {
  const unsigned T = add_threads();
  i1.resize(n);
  i2.resize(n);
  const PartOwner owner(T);
  HostVec<uint8_t> pa(n), pb(n, 0xff);  // role B (node pairs) is checked on the GPU
  std::vector<size_t> tmiss(T, n);
  std::vector<uint32_t> tmax(T, 0);
  parallel_chunks(T, n, [&](unsigned t, size_t b, size_t e) {
    uint32_t mx = 0;
    for (size_t q = b; q < e; ++q) {
      const int64_t a = h->node_idx.find(nodes[2 * q]), c = h->node_idx.find(nodes[2 * q + 1]);
      if ((a < 0 || c < 0) && tmiss[t] == n) tmiss[t] = q;
      i1[q] = (int32_t)a;
      i2[q] = (int32_t)c;
      mx = std::max(mx, numbers[q]);
    }
    tmax[t] = mx;
  });
  const size_t limit = *std::min_element(tmiss.begin(), tmiss.end());
  // the node indexes of the items before the first missing node go up now: the GPU checks their pairs
  // against every element's of the kind while the host checks the numbers
  CK(upload(dn1, base, i1.data(), limit, h->stream));
  CK(upload(dn2, base, i2.data(), limit, h->stream));
  const size_t total = base + limit;
  const int32_t *d1 = dn1.p, *d2 = dn2.p;
  DupSearch dup;
  int st = dup_start(
      h, dup, total,
      [&](unsigned long long* key, uint32_t* idx) {
        k_pair_keys<<<grid_for(total, 256), 256, 0, h->stream>>>(total, d1, d2, key, idx);
      },
      [&](const unsigned long long* skey, const uint32_t* sidx, unsigned long long* out) {
        k_pair_dups<<<grid_for(total, 256), 256, 0, h->stream>>>(total, skey, sidx, out);
      });
  if (st) return st;
  by_num.fit(*std::max_element(tmax.begin(), tmax.end()));
  parallel_chunks(T, n, [&](unsigned, size_t b, size_t e) {
    for (size_t q = b; q < e; ++q) pa[q] = owner.of_part(by_num.part(numbers[q]));
  });
  int role = 0;
  size_t f = registry_pass(
      T, limit, pa.data(), pb.data(),
      [&](size_t q) {
        if (by_num.find(numbers[q]) >= 0) return false;
        by_num.insert(numbers[q], (int64_t)(base + q));
        return true;
      },
      [&](size_t) { return true; }, [&](size_t q) { by_num.prefetch(numbers[q]); }, [&](size_t) {}, &role);
  size_t fp = total;
  st = dup_finish(h, dup, &fp);
  if (st) return st;
  if (fp >= base && fp - base < f) {  // (the model's elements have distinct pairs: fp < base cannot happen)
    f = fp - base;
    role = 2;
  }
  for (size_t q = f; q < limit; ++q) by_num.erase(numbers[q], (int64_t)(base + q));
  i1.resize(f);
  i2.resize(f);
  *passed = f;
  if (f == n) return FEM_GPU_OK;
  if (role == 1) return h->fail(FEM_GPU_ERR_ELEM_NUMBER, "%s element with number %u already exists!", kind, numbers[f]);
  if (role == 2)
    return h->fail(FEM_GPU_ERR_ELEM_SAME_NODES, "%s element with node number %u and %u already exists!", kind,
                   nodes[2 * f], nodes[2 * f + 1]);
  int32_t idx;
  const int c = lookup_node(h, nodes[2 * f], &idx);
  return c ? c : lookup_node(h, nodes[2 * f + 1], &idx);
}

// The same for plates: the four nodes exist, the number is new, the node set is new.  Returns -1
// (nothing changed) when an item before the first missing node repeats a node number: those take
// the sequential loop's subset test.
// (props: young, poisson, thickness, shear factor of the call's plates; *validated gets the number of items
// whose validation kernel was started here -- it runs on the GPU while the host checks the numbers)
int plate_checks(fem_gpu* h, const uint32_t* numbers, const uint32_t* nodes, size_t n, HostVec<int32_t>* id,
                 size_t* passed, const double* const props[4], size_t* validated) {
  const unsigned T = add_threads();
  const size_t base = h->np;
  for (int q = 0; q < 4; ++q) id[q].resize(n);
  const PartOwner owner(T);
  HostVec<uint8_t> pa(n), pb(n, 0xff);  // role B (node sets) is checked on the GPU
  std::vector<size_t> tmiss(T, n), trep(T, n);
  std::vector<uint32_t> tmax(T, 0);
  parallel_chunks(T, n, [&](unsigned t, size_t b, size_t e) {
    uint32_t mx = 0;
    for (size_t q = b; q < e; ++q) {
      const uint32_t* nn = nodes + 4 * q;
      bool miss = false;
      for (int c = 0; c < 4; ++c) {
        const int64_t i = h->node_idx.find(nn[c]);
        miss = miss || i < 0;
        id[c][q] = (int32_t)i;
      }
      if (miss && tmiss[t] == n) tmiss[t] = q;
      const Set4 key = sorted4(nn);
      if ((key.s[0] == key.s[1] || key.s[1] == key.s[2] || key.s[2] == key.s[3]) && trep[t] == n) trep[t] = q;
      mx = std::max(mx, numbers[q]);
    }
    tmax[t] = mx;
  });
  const size_t limit = *std::min_element(tmiss.begin(), tmiss.end());
  if (*std::min_element(trep.begin(), trep.end()) < limit) return -1;
  // the node indexes of the items before the first missing node go up now: the GPU checks their node sets
  // against every plate's while the host checks the numbers
  for (int c = 0; c < 4; ++c) {
    DevBuf<int32_t>& dst = c == 0 ? h->p_n1 : c == 1 ? h->p_n2 : c == 2 ? h->p_n3 : h->p_n4;
    CK(upload(dst, base, id[c].data(), limit, h->stream));
  }
  // their properties too, and the validation of these items starts now (it needs no host check)
  CK(upload(h->p_E, base, props[0], limit, h->stream));
  CK(upload(h->p_nu, base, props[1], limit, h->stream));
  CK(upload(h->p_t, base, props[2], limit, h->stream));
  CK(upload(h->p_ks, base, props[3], limit, h->stream));
  {
    const NodesView nd = h->nodes();
    const PlateView pv = h->plates();
    const double abs_tol = h->abs_tol;
    int vs = validate_start(h, limit, [&](int* s_, unsigned long long* f_) {
      k_validate_plate<<<grid_for(limit, 128), 128, 0, h->stream>>>(nd, pv, abs_tol, base, limit, s_, f_);
    });
    if (vs) return vs;
    *validated = limit;
  }
  const size_t total = base + limit;
  const int32_t *n1 = h->p_n1.p, *n2 = h->p_n2.p, *n3 = h->p_n3.p, *n4 = h->p_n4.p;
  DupSearch dup;
  int st = dup_start(
      h, dup, total,
      [&](unsigned long long* key, uint32_t* idx) {
        k_set4_keys<<<grid_for(total, 256), 256, 0, h->stream>>>(total, n1, n2, n3, n4, key, idx);
      },
      [&](const unsigned long long* skey, const uint32_t* sidx, unsigned long long* out) {
        k_set4_dups<<<grid_for(total, 256), 256, 0, h->stream>>>(total, skey, sidx, n1, n2, n3, n4, out);
      });
  if (st) return st;
  h->p_by_num.fit(*std::max_element(tmax.begin(), tmax.end()));
  parallel_chunks(T, n, [&](unsigned, size_t b, size_t e) {
    for (size_t q = b; q < e; ++q) pa[q] = owner.of_part(h->p_by_num.part(numbers[q]));
  });
  int role = 0;
  size_t f = registry_pass(
      T, limit, pa.data(), pb.data(),
      [&](size_t q) {
        if (h->p_by_num.find(numbers[q]) >= 0) return false;
        h->p_by_num.insert(numbers[q], (int64_t)(base + q));
        return true;
      },
      [&](size_t) { return true; }, [&](size_t q) { h->p_by_num.prefetch(numbers[q]); }, [&](size_t) {}, &role);
  size_t fs = total;
  st = dup_finish(h, dup, &fs);
  if (st) return st;
  if (fs >= base && fs - base < f) {  // (the model's plates have distinct node sets: fs < base cannot happen)
    f = fs - base;
    role = 2;
  }
  for (size_t q = f; q < limit; ++q) h->p_by_num.erase(numbers[q], (int64_t)(base + q));
  for (int c = 0; c < 4; ++c) id[c].resize(f);
  *passed = f;
  if (f == n) return FEM_GPU_OK;
  const uint32_t* nn = nodes + 4 * f;
  if (role == 1) return h->fail(FEM_GPU_ERR_ELEM_NUMBER, "Plate element with number %u already exists!", numbers[f]);
  if (role == 2)
    return h->fail(FEM_GPU_ERR_ELEM_SAME_NODES, "Plate element with nodes numbers [%u, %u, %u, %u] already exists!",
                   nn[0], nn[1], nn[2], nn[3]);
  int32_t idx;
  for (int c = 0; c < 4; ++c) {
    const int sl = lookup_node(h, nn[c], &idx);
    if (sl) return sl;
  }
  return FEM_GPU_OK;
}
}  // namespace

// add_truss, methods_for_truss_data_handle.rs:32-128 and structs/truss.rs:44-64
extern "C" int fem_gpu_add_trusses(fem_gpu_t* h, const uint32_t* numbers, const uint32_t* nodes, const double* young,
                                   const double* area, const double* area2, size_t n, size_t* n_added) {
  if (n_added) *n_added = 0;
  if (!h || (n && (!numbers || !nodes || !young || !area))) return FEM_GPU_ERR_ARGUMENT;
  int st = ensure_ready(h);
  if (st) return st;
  h->drop_numeric_graph();  // the element and node arrays may move
  HostVec<int32_t> i1, i2;
  HostVec<double> a2v;
  i1.reserve(n);
  i2.reserve(n);
  a2v.reserve(n);
  int host_code = FEM_GPU_OK;
  std::string host_err;
  size_t k = 0;
  h->t_by_num.reserve(h->nt + n);
  const bool bulk = n >= kParallelAdd;
  if (bulk) {
    host_code = two_node_checks(h, "Truss", h->t_by_num, h->t_n1, h->t_n2, h->nt, numbers, nodes, n, i1, i2, &k);
    if (host_code >= FEM_GPU_ERR_CUDA) return host_code;
    a2v.resize(k);
    for (size_t q = 0; q < k; ++q) a2v[q] = area2 ? area2[q] : NAN;
  }
  if (!bulk) {
    ensure_pairs(h->t_pairs, &h->t_pairs_built, h->nt, h->t_nodes);
    h->t_pairs.reserve(h->nt + n);
  }
  for (; k < n && !bulk; ++k) {
    if (k + kRegAhead < n) {
      const uint32_t* f = nodes + 2 * (k + kRegAhead);
      h->t_pairs.prefetch(pair_key(f[0], f[1]));
      h->node_idx.prefetch(f[0]);
      h->node_idx.prefetch(f[1]);
    }
    uint32_t num = numbers[k], u = nodes[2 * k], v = nodes[2 * k + 1];
    int32_t a, b;
    if ((host_code = lookup_node(h, u, &a)) || (host_code = lookup_node(h, v, &b))) break;
    if (h->t_by_num.find(num) >= 0) {
      host_code = h->fail(FEM_GPU_ERR_ELEM_NUMBER, "Truss element with number %u already exists!", num);
      break;
    }
    if (h->t_pairs.find(pair_key(u, v)) >= 0) {
      host_code = h->fail(FEM_GPU_ERR_ELEM_SAME_NODES, "Truss element with node number %u and %u already exists!", u, v);
      break;
    }
    h->t_by_num.insert(num, (int64_t)(h->nt + k));
    h->t_pairs.insert(pair_key(u, v), (int64_t)(h->nt + k));
    i1.push_back(a);
    i2.push_back(b);
    a2v.push_back(area2 ? area2[k] : NAN);
  }
  if (host_code) host_err = h->err;
  size_t m = k, base = h->nt;
  if (!bulk) {  // (the bulk checks sent the node indexes up already)
    CK(upload(h->t_n1, base, i1.data(), m, h->stream));
    CK(upload(h->t_n2, base, i2.data(), m, h->stream));
  }
  CK(upload(h->t_E, base, young, m, h->stream));
  CK(upload(h->t_A, base, area, m, h->stream));
  CK(upload(h->t_A2, base, a2v.data(), m, h->stream));
  size_t bad;
  int code;
  NodesView nd = h->nodes();
  int32_t *n1 = h->t_n1.p, *n2 = h->t_n2.p;
  double *E = h->t_E.p, *A = h->t_A.p, *A2 = h->t_A2.p;
  st = first_failure(
      h, m,
      [&](int* s, unsigned long long* f) {
        k_validate_truss<<<grid_for(m, 128), 128, 0, h->stream>>>(nd, n1, n2, E, A, A2, base, m, s, f);
      },
      [&] {  // the host arrays take every item now and drop the rejected ones after the result
        append_host(h->t_num, numbers, m);
        append_host(h->t_nodes, nodes, 2 * m);
      },
      &bad, &code);
  size_t accepted = st ? 0 : std::min(m, bad);
  h->t_num.resize(base + accepted);
  h->t_nodes.resize(2 * (base + accepted));
  if (st) return st;
  for (size_t j = accepted; j < m; ++j) {  // roll back registry entries past the failure
    h->t_by_num.erase(numbers[j], (int64_t)(base + j));
    if (!bulk) h->t_pairs.erase(pair_key(nodes[2 * j], nodes[2 * j + 1]), (int64_t)(base + j));
  }
  h->nt += accepted;
  if (!bulk) h->t_pairs_built = h->nt;
  h->append_run(kTruss, base, accepted);
  if (n_added) *n_added = accepted;
  if (bad < m) {
    char b[48];
    switch (code) {
      case FEM_GPU_ERR_YOUNG:
        return h->fail(code, "Young's modulus %s is less or equal to zero!", rust_f64(young[bad]).c_str());
      case FEM_GPU_ERR_AREA: return h->fail(code, "Area %s is less or equal to zero!", rust_f64(area[bad]).c_str());
      case FEM_GPU_ERR_AREA2:
        return h->fail(code, "Area2 %s is less or equal to zero!", rust_f64(area2[bad]).c_str());
      default:
        snprintf(b, sizeof b, "%u", numbers[bad]);
        return h->fail(code, "Truss element %s has coincident nodes %u and %u!", b, nodes[2 * bad], nodes[2 * bad + 1]);
    }
  }
  if (host_code) {
    h->err = host_err;
    return host_code;
  }
  return FEM_GPU_OK;
}

// add_beam, methods_for_beam_data_handle.rs:32-142 and structs/beam.rs:63-117
extern "C" int fem_gpu_add_beams(fem_gpu_t* h, const uint32_t* numbers, const uint32_t* nodes, const double* young,
                                 const double* poisson, const double* area, const double* i11, const double* i22,
                                 const double* i12, const double* it, const double* shear_factor,
                                 const double* local_axis, size_t n, size_t* n_added) {
  if (n_added) *n_added = 0;
  if (!h || (n && (!numbers || !nodes || !young || !poisson || !area || !i11 || !i22 || !i12 || !it ||
                   !shear_factor || !local_axis)))
    return FEM_GPU_ERR_ARGUMENT;
  int st = ensure_ready(h);
  if (st) return st;
  h->drop_numeric_graph();  // the element and node arrays may move
  HostVec<int32_t> i1, i2;
  HostVec<double> ax, ay, az;
  int host_code = FEM_GPU_OK;
  std::string host_err;
  size_t k = 0;
  h->b_by_num.reserve(h->nbm + n);
  const bool bulk = n >= kParallelAdd;
  i1.reserve(n);
  i2.reserve(n);
  ax.reserve(n);
  ay.reserve(n);
  az.reserve(n);
  if (bulk) {
    host_code = two_node_checks(h, "Beam", h->b_by_num, h->b_n1, h->b_n2, h->nbm, numbers, nodes, n, i1, i2, &k);
    if (host_code >= FEM_GPU_ERR_CUDA) return host_code;
    ax.resize(k);
    ay.resize(k);
    az.resize(k);
    parallel_chunks(add_threads(), k, [&](unsigned, size_t b, size_t e) {
      for (size_t q = b; q < e; ++q) {
        ax[q] = local_axis[3 * q];
        ay[q] = local_axis[3 * q + 1];
        az[q] = local_axis[3 * q + 2];
      }
    });
  }
  if (!bulk) {
    ensure_pairs(h->b_pairs, &h->b_pairs_built, h->nbm, h->b_nodes);
    h->b_pairs.reserve(h->nbm + n);
  }
  for (; k < n && !bulk; ++k) {
    if (k + kRegAhead < n) {
      const uint32_t* f = nodes + 2 * (k + kRegAhead);
      h->b_pairs.prefetch(pair_key(f[0], f[1]));
      h->node_idx.prefetch(f[0]);
      h->node_idx.prefetch(f[1]);
    }
    uint32_t num = numbers[k], u = nodes[2 * k], v = nodes[2 * k + 1];
    int32_t a, b;
    if ((host_code = lookup_node(h, u, &a)) || (host_code = lookup_node(h, v, &b))) break;
    if (h->b_by_num.find(num) >= 0) {
      host_code = h->fail(FEM_GPU_ERR_ELEM_NUMBER, "Beam element with number %u already exists!", num);
      break;
    }
    if (h->b_pairs.find(pair_key(u, v)) >= 0) {
      host_code = h->fail(FEM_GPU_ERR_ELEM_SAME_NODES, "Beam element with node number %u and %u already exists!", u, v);
      break;
    }
    h->b_by_num.insert(num, (int64_t)(h->nbm + k));
    h->b_pairs.insert(pair_key(u, v), (int64_t)(h->nbm + k));
    i1.push_back(a);
    i2.push_back(b);
    ax.push_back(local_axis[3 * k]);
    ay.push_back(local_axis[3 * k + 1]);
    az.push_back(local_axis[3 * k + 2]);
  }
  if (host_code) host_err = h->err;
  size_t m = k, base = h->nbm;
  if (!bulk) {  // (the bulk checks sent the node indexes up already)
    CK(upload(h->b_n1, base, i1.data(), m, h->stream));
    CK(upload(h->b_n2, base, i2.data(), m, h->stream));
  }
  CK(upload(h->b_E, base, young, m, h->stream));
  CK(upload(h->b_nu, base, poisson, m, h->stream));
  CK(upload(h->b_A, base, area, m, h->stream));
  CK(upload(h->b_i11, base, i11, m, h->stream));
  CK(upload(h->b_i22, base, i22, m, h->stream));
  CK(upload(h->b_i12, base, i12, m, h->stream));
  CK(upload(h->b_it, base, it, m, h->stream));
  CK(upload(h->b_ks, base, shear_factor, m, h->stream));
  CK(upload(h->b_ax, base, ax.data(), m, h->stream));
  CK(upload(h->b_ay, base, ay.data(), m, h->stream));
  CK(upload(h->b_az, base, az.data(), m, h->stream));
  size_t bad;
  int code;
  NodesView nd = h->nodes();
  BeamView bv = h->beams();
  st = first_failure(
      h, m,
      [&](int* s, unsigned long long* f) {
        k_validate_beam<<<grid_for(m, 128), 128, 0, h->stream>>>(nd, bv, base, m, s, f);
      },
      [&] {  // the host arrays take every item now and drop the rejected ones after the result
        append_host(h->b_num, numbers, m);
        append_host(h->b_nodes, nodes, 2 * m);
      },
      &bad, &code);
  size_t accepted = st ? 0 : std::min(m, bad);
  h->b_num.resize(base + accepted);
  h->b_nodes.resize(2 * (base + accepted));
  if (st) return st;
  for (size_t j = accepted; j < m; ++j) {
    h->b_by_num.erase(numbers[j], (int64_t)(base + j));
    if (!bulk) h->b_pairs.erase(pair_key(nodes[2 * j], nodes[2 * j + 1]), (int64_t)(base + j));
  }
  h->nbm += accepted;
  if (!bulk) h->b_pairs_built = h->nbm;
  h->append_run(kBeam, base, accepted);
  if (n_added) *n_added = accepted;
  if (bad < m) {
    switch (code) {
      case FEM_GPU_ERR_YOUNG:
        return h->fail(code, "Young's modulus %s is less or equal to zero!", rust_f64(young[bad]).c_str());
      case FEM_GPU_ERR_POISSON:  // beam.rs:84 reports the Young's modulus value
        return h->fail(code, "Poisson's ratio %s is less or equal to zero!", rust_f64(young[bad]).c_str());
      case FEM_GPU_ERR_AREA: return h->fail(code, "Area %s is less or equal to zero!", rust_f64(area[bad]).c_str());
      case FEM_GPU_ERR_I11: return h->fail(code, "I11 %s is less or equal to zero!", rust_f64(i11[bad]).c_str());
      case FEM_GPU_ERR_I22: return h->fail(code, "I22 %s is less or equal to zero!", rust_f64(i22[bad]).c_str());
      case FEM_GPU_ERR_IT: return h->fail(code, "It %s is less or equal to zero!", rust_f64(it[bad]).c_str());
      case FEM_GPU_ERR_SHEAR_FACTOR:
        return h->fail(code, "Shear factor %s is less or equal to zero!", rust_f64(shear_factor[bad]).c_str());
      case FEM_GPU_ERR_PARALLEL_AXIS:
        return h->fail(code, "Local axis 1 direction [%s, %s, %s] parallel to element %u!",
                       rust_f64(local_axis[3 * bad]).c_str(), rust_f64(local_axis[3 * bad + 1]).c_str(),
                       rust_f64(local_axis[3 * bad + 2]).c_str(), numbers[bad]);
      default:
        return h->fail(code, "Beam element %u has coincident nodes %u and %u!", numbers[bad], nodes[2 * bad],
                       nodes[2 * bad + 1]);
    }
  }
  if (host_code) {
    h->err = host_err;
    return host_code;
  }
  return FEM_GPU_OK;
}

// add_plate, methods_for_plate_data_handle.rs:33-217 and structs/plate.rs:58-158
extern "C" int fem_gpu_add_plates(fem_gpu_t* h, const uint32_t* numbers, const uint32_t* nodes, const double* young,
                                  const double* poisson, const double* thickness, const double* shear_factor,
                                  size_t n, size_t* n_added) {
  if (n_added) *n_added = 0;
  if (!h || (n && (!numbers || !nodes || !young || !poisson || !thickness || !shear_factor)))
    return FEM_GPU_ERR_ARGUMENT;
  int st = ensure_ready(h);
  if (st) return st;
  h->drop_numeric_graph();  // the element and node arrays may move
  HostVec<int32_t> id[4];
  for (auto& v : id) v.reserve(n);
  int host_code = FEM_GPU_OK;
  std::string host_err;
  size_t k = 0;
  h->p_by_num.reserve(h->np + n);
  h->p_nodes.reserve(4 * (h->np + n));
  h->p_num.reserve(h->np + n);
  bool sequential = n < kParallelAdd;
  size_t validated = 0;  // items whose validation the bulk checks started
  if (!sequential) {
    const double* const props[4] = {young, poisson, thickness, shear_factor};
    host_code = plate_checks(h, numbers, nodes, n, id, &k, props, &validated);
    if (host_code < 0) {  // repeated node numbers: the sequential loop's subset test
      host_code = FEM_GPU_OK;
      sequential = true;
      k = 0;
      for (auto& v : id) v.clear();
    } else if (host_code >= FEM_GPU_ERR_CUDA) {
      return host_code;
    }
  }
  if (sequential) {
    ensure_sets(h);
    h->p_sets.reserve(h->np + n);
  }
  for (; k < n && sequential; ++k) {
    if (k + kRegAhead < n) {
      const uint32_t* f = nodes + 4 * (k + kRegAhead);
      h->p_sets.prefetch(set4_hash(sorted4(f)));
      for (int q = 0; q < 4; ++q) h->node_idx.prefetch(f[q]);
    }
    uint32_t num = numbers[k];
    const uint32_t* nn = nodes + 4 * k;
    int32_t ix[4];
    bool okn = true;
    for (int q = 0; q < 4 && okn; ++q)
      if ((host_code = lookup_node(h, nn[q], &ix[q]))) okn = false;
    if (!okn) break;
    if (h->p_by_num.find(num) >= 0) {
      host_code = h->fail(FEM_GPU_ERR_ELEM_NUMBER, "Plate element with number %u already exists!", num);
      break;
    }
    // Plate::is_nodes_numbers_same (plate.rs:1107-1118): every given number belongs to an existing plate
    bool distinct = nn[0] != nn[1] && nn[0] != nn[2] && nn[0] != nn[3] && nn[1] != nn[2] && nn[1] != nn[3] &&
                    nn[2] != nn[3];
    bool same = false;
    if (distinct) {
      const Set4 key = sorted4(nn);
      const size_t np0 = h->np;
      same = h->p_sets.find(set4_hash(key), [&](int64_t e) {
        const uint32_t* mm = (size_t)e < np0 ? &h->p_nodes[4 * (size_t)e] : nodes + 4 * ((size_t)e - np0);
        return sorted4(mm) == key;
      }) >= 0;
    } else {
      for (size_t e = 0; e < h->p_num.size() + k && !same; ++e) {
        const uint32_t* mm = e < h->p_num.size() ? &h->p_nodes[4 * e] : nodes + 4 * (e - h->p_num.size());
        bool all = true;
        for (int q = 0; q < 4 && all; ++q) all = nn[q] == mm[0] || nn[q] == mm[1] || nn[q] == mm[2] || nn[q] == mm[3];
        same = all;
      }
    }
    if (same) {
      host_code = h->fail(FEM_GPU_ERR_ELEM_SAME_NODES, "Plate element with nodes numbers [%u, %u, %u, %u] already exists!",
                          nn[0], nn[1], nn[2], nn[3]);
      break;
    }
    h->p_by_num.insert(num, (int64_t)(h->np + k));
    h->p_sets.insert(set4_hash(sorted4(nn)), (int64_t)(h->np + k));
    for (int q = 0; q < 4; ++q) id[q].push_back(ix[q]);
  }
  if (host_code) host_err = h->err;
  size_t m = k, base = h->np;
  if (sequential) {  // (the bulk checks sent the node indexes up already)
    CK(upload(h->p_n1, base, id[0].data(), m, h->stream));
    CK(upload(h->p_n2, base, id[1].data(), m, h->stream));
    CK(upload(h->p_n3, base, id[2].data(), m, h->stream));
    CK(upload(h->p_n4, base, id[3].data(), m, h->stream));
  }
  size_t bad;
  int code;
  if (validated >= m) {  // the bulk checks started the validation of these items already
    append_host(h->p_num, numbers, m);  // the host arrays take every item now and drop the rejected ones after
    append_host(h->p_nodes, nodes, 4 * m);
    st = validate_finish(h, m, &bad, &code);
  } else {
    CK(upload(h->p_E, base, young, m, h->stream));
    CK(upload(h->p_nu, base, poisson, m, h->stream));
    CK(upload(h->p_t, base, thickness, m, h->stream));
    CK(upload(h->p_ks, base, shear_factor, m, h->stream));
    NodesView nd = h->nodes();
    PlateView pv = h->plates();
    double abs_tol = h->abs_tol;
    st = first_failure(
        h, m,
        [&](int* s, unsigned long long* f) {
          k_validate_plate<<<grid_for(m, 128), 128, 0, h->stream>>>(nd, pv, abs_tol, base, m, s, f);
        },
        [&] {  // the host arrays take every item now and drop the rejected ones after the result
          append_host(h->p_num, numbers, m);
          append_host(h->p_nodes, nodes, 4 * m);
        },
        &bad, &code);
  }
  size_t accepted = st ? 0 : std::min(m, bad);
  h->p_num.resize(base + accepted);
  h->p_nodes.resize(4 * (base + accepted));
  if (st) return st;
  for (size_t j = accepted; j < m; ++j) {
    h->p_by_num.erase(numbers[j], (int64_t)(base + j));
    if (sequential) h->p_sets.erase(set4_hash(sorted4(nodes + 4 * j)), (int64_t)(base + j));
  }
  h->np += accepted;
  if (sequential) h->sets_built = h->np;
  h->append_run(kPlate, base, accepted);
  if (n_added) *n_added = accepted;
  if (bad < m) {
    switch (code) {
      case FEM_GPU_ERR_YOUNG:
        return h->fail(code, "Young's modulus %s is less or equal to zero!", rust_f64(young[bad]).c_str());
      case FEM_GPU_ERR_POISSON:  // plate.rs:79 reports the Young's modulus value
        return h->fail(code, "Poisson's ratio %s is less or equal to zero!", rust_f64(young[bad]).c_str());
      case FEM_GPU_ERR_THICKNESS:  // plate.rs:82 reports the Young's modulus value
        return h->fail(code, "Thickness %s is less or equal to zero!", rust_f64(young[bad]).c_str());
      case FEM_GPU_ERR_SHEAR_FACTOR:
        return h->fail(code, "Shear factor %s is less or equal to zero!", rust_f64(shear_factor[bad]).c_str());
      case FEM_GPU_ERR_NODES_ON_LINE: return h->fail(code, "Some nodes of %u element lie on the line!", numbers[bad]);
      case FEM_GPU_ERR_NOT_ON_PLANE: return h->fail(code, "Not all nodes of element %u lie on the plane!", numbers[bad]);
      default: return h->fail(code, "Element %u non-convex!", numbers[bad]);
    }
  }
  if (host_code) {
    h->err = host_err;
    return host_code;
  }
  return FEM_GPU_OK;
}

namespace {

int launch_elements(fem_gpu* h, BlockSink sink_t, BlockSink sink_b, BlockSink sink_p) {
  NodesView nd = h->nodes();
  if (h->nt)
    k_truss<<<grid_for(h->nt, 128), 128, 0, h->stream>>>(nd, h->trusses(), h->abs_tol, h->nt, sink_t);
  if (h->nbm)
    k_beam<<<grid_for(h->nbm, 128), 128, 0, h->stream>>>(nd, h->beams(), h->rel_tol, h->abs_tol, h->nbm, sink_b);
  if (h->np)
    k_plate<<<grid_for(h->np, FEM_PLATE_BLOCK), FEM_PLATE_BLOCK, plate_smem(sink_p, FEM_PLATE_BLOCK), h->stream>>>(
        nd, h->plates(), h->abs_tol, h->np, sink_p);
  CK(cudaGetLastError());
  return FEM_GPU_OK;
}

// the numeric pass's operations (captured into the handle's graph); the phase events are graph nodes
int numeric_enqueue(fem_gpu* h, bool captured) {
  // phase events: graph nodes when captured, plain records otherwise
  auto mark = [&](cudaEvent_t ev) {
    return captured ? cudaEventRecordWithFlags(ev, h->stream, cudaEventRecordExternal) : cudaEventRecord(ev, h->stream);
  };
  CK(cudaMemsetAsync(h->flag.p, 0, sizeof(int), h->stream));
  CK(mark(h->ev[0]));
  BlockSink st{nullptr, h->V.p, h->off_t.p, h->flag.p, h->v_words};
  BlockSink sb{nullptr, h->V.p, h->off_b.p, h->flag.p, h->v_words};
  BlockSink sp{nullptr, h->V.p, h->off_p.p, h->flag.p, h->v_words};
  int r = launch_elements(h, st, sb, sp);
  if (r) return r;
  CK(mark(h->ev[1]));
  if (h->n_blocks) {
    if (h->n_desc)
      k_block_sums<<<block_sums_grid(h->n_desc, 256), 256, 0, h->stream>>>(h->n_desc, h->s_words, h->slot_desc.p, h->V.p,
                                                                     h->V.p + h->vs_off, h->flag.p, h->v_words);
    k_gather_values<<<grid_for(((size_t)h->nnz + kGatherPerThread - 1) / kGatherPerThread, 256), 256, 0,
                      h->stream>>>((size_t)h->nnz, h->src_map.p, h->V.p, h->vs_off, h->values.p, h->flag.p,
                                   h->vs_off + h->s_words);
  }
  CK(cudaGetLastError());
  CK(mark(h->ev[2]));
  return FEM_GPU_OK;
}

// One numeric pass: the first after a symbolic phase runs its kernels directly, later ones are a single graph
// launch (the pass's arrays keep their addresses until the next
// symbolic phase, which drops the graph)
int numeric_launch(fem_gpu* h) {
  h->sep_valid = false;  // a separation describes the stiffness it was taken from
  h->sell_valid = false;
  if (!h->num_graph && !h->num_eager_done) {
    // the first pass after a symbolic phase runs its kernels directly: capturing and instantiating the
    // graph costs host time the single assemble of a new model would wait for; the next pass captures it
    h->num_eager_done = true;
    const int r = numeric_enqueue(h, false);
    if (r) return r;
    h->numeric_done = true;
    return FEM_GPU_OK;
  }
  if (!h->num_graph) {
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    const int r = numeric_enqueue(h, true);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    if (r) {
      if (g) cudaGraphDestroy(g);
      return r;
    }
    if (e != cudaSuccess) return h->cuda_fail(e, "cudaStreamEndCapture");
    const cudaError_t ei = cudaGraphInstantiate(&h->num_graph, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
      h->num_graph = nullptr;
      return h->cuda_fail(ei, "cudaGraphInstantiate");
    }
  }
  CK(cudaGraphLaunch(h->num_graph, h->stream));
  h->numeric_done = true;
  return FEM_GPU_OK;
}


// Host buffers a caller wants the pattern read back into (fem_gpu_assemble_to_host): the symbolic phase sends
// row_ptr back once the rows are counted and the columns in node chunks as the row fill finishes each, on the
// copy stream, so the host link starts on the pattern before the phase ends.
struct PatternCopy {
  int64_t* row_ptr;
  int32_t* col_idx;
  int64_t capacity;     // entries col_idx has room for (nothing is sent when the pattern is larger)
  bool issued = false;  // set when the copies were enqueued
};
constexpr int kFillChunks = 4;
const char* const kTooManyMsg = "a node pair is shared by 2^24 or more elements";

int symbolic(fem_gpu* h, PatternCopy* pc = nullptr) {
  h->drop_numeric_graph();
  cudaStream_t s = h->stream;
  size_t np = h->n_pairs;
  const size_t nrows = (size_t)h->nodes_number * 6;
  CK(h->row_ptr.reserve(nrows + 1, s));
  h->n_blocks = 0;
  h->nnz = 0;
  h->n_groups = 0;
  if (np == 0) {
    CK(cudaMemsetAsync(h->row_ptr.p, 0, (nrows + 1) * sizeof(int64_t), s));
    CK(cudaStreamSynchronize(s));
    h->pattern_valid = true;
    return FEM_GPU_OK;
  }
  // bits of the largest node index (keys pack two indices in 2 kb bits)
  int kb = 1;
  while (kb < 32 && (((uint64_t)h->nodes_number - 1) >> kb) != 0) ++kb;
  // 1. pair keys in call order
  DevBuf<uint64_t> keys, skeys;
  DevBuf<uint32_t> vals, svals;
  CK(keys.reserve(np, s));
  CK(skeys.reserve(np, s));
  CK(vals.reserve(np, s));
  CK(svals.reserve(np, s));
  for (const Run& r : h->runs) {
    if (r.kind == kTruss)
      k_gen_pairs<<<grid_for(r.count, 256), 256, 0, s>>>(kTruss, h->t_n1.p, h->t_n2.p, nullptr, nullptr, r.begin,
                                                         r.count, r.pair_base, kb, keys.p, vals.p);
    else if (r.kind == kBeam)
      k_gen_pairs<<<grid_for(r.count, 256), 256, 0, s>>>(kBeam, h->b_n1.p, h->b_n2.p, nullptr, nullptr, r.begin,
                                                         r.count, r.pair_base, kb, keys.p, vals.p);
    else
      k_gen_pairs<<<grid_for(r.count, 256), 256, 0, s>>>(kPlate, h->p_n1.p, h->p_n2.p, h->p_n3.p, h->p_n4.p,
                                                         r.begin, r.count, r.pair_base, kb, keys.p, vals.p);
  }
  CK(cudaGetLastError());
  // 2. per-pair non-zero masks from the element arithmetic
  CK(h->mask_t.reserve(h->nt * kPairs2 + 1, s));
  CK(h->mask_b.reserve(h->nbm * kPairs2 + 1, s));
  CK(h->mask_p.reserve(h->np * kPairs4 + 1, s));
  {
    BlockSink st{h->mask_t.p, nullptr, nullptr, nullptr};
    BlockSink sb{h->mask_b.p, nullptr, nullptr, nullptr};
    BlockSink sp{h->mask_p.p, nullptr, nullptr, nullptr};
    int r = launch_elements(h, st, sb, sp);
    if (r) return r;
  }
  // 3. stable sort by node-pair key (call order preserved within a block)
  int st = cub_call(h, [&](void* tmp, size_t& bytes) {
    return cub::DeviceRadixSort::SortPairs(tmp, bytes, keys.p, skeys.p, vals.p, svals.p, (int64_t)np, 0, 2 * kb, s);
  });
  if (st) return st;
  // 4. slots and sorted masks
  CK(h->slot_t.reserve(h->nt * kPairs2 + 1, s));
  CK(h->slot_b.reserve(h->nbm * kPairs2 + 1, s));
  CK(h->slot_p.reserve(h->np * kPairs4 + 1, s));
  DevBuf<uint64_t> smask;
  CK(smask.reserve(np, s));
  k_scatter_slots<<<grid_for(np, 256), 256, 0, s>>>(svals.p, np, h->slot_t.p, h->slot_b.p, h->slot_p.p, h->mask_t.p,
                                                     h->mask_b.p, h->mask_p.p, smask.p);
  // 5. blocks
  DevBuf<uint32_t> head, incl;
  CK(head.reserve(np, s));
  CK(incl.reserve(np, s));
  k_heads<<<grid_for(np, 256), 256, 0, s>>>(skeys.p, np, head.p);
  st = cub_call(h, [&](void* tmp, size_t& bytes) {
    return cub::DeviceScan::InclusiveSum(tmp, bytes, head.p, incl.p, (int64_t)np, s);
  });
  if (st) return st;
  uint32_t nb32 = 0;
  CK(cudaMemcpyAsync(&nb32, incl.p + np - 1, sizeof nb32, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  size_t nb = nb32;
  h->n_blocks = nb;
  CK(h->blk_start.reserve(nb, s));
  CK(h->blk_count.reserve(nb, s));
  CK(h->blk_mask.reserve(nb, s));
  CK(h->blk_maskT.reserve(nb, s));
  CK(h->blk_I.reserve(nb, s));
  CK(h->blk_J.reserve(nb, s));
  k_block_starts<<<grid_for(np, 256), 256, 0, s>>>(incl.p, np, h->blk_start.p);
  k_block_meta<<<grid_for(nb, 256), 256, 0, s>>>(h->blk_start.p, nb, np, skeys.p, kb, smask.p, h->blk_count.p,
                                                 h->blk_mask.p, h->blk_maskT.p, h->blk_I.p, h->blk_J.p);
  // compacted scratch: block offsets and, per element pair, its offset and mask
  {
    DevBuf<unsigned long long> sizes;
    CK(sizes.reserve(nb + 2, s));
    CK(h->blk_voff.reserve(nb + 1, s));
    CK(h->blk_lay.reserve(nb + 1, s));
    CK(cudaMemsetAsync(sizes.p + nb, 0, 2 * sizeof(unsigned long long), s));  // the scan's tail, the padding count
    CK(h->blk_pmask.reserve(nb + 1, s));
    k_block_sizes<<<grid_for(nb, 256), 256, 0, s>>>(nb, h->blk_count.p, h->blk_mask.p, h->blk_I.p, h->blk_J.p,
                                                    h->blk_lay.p, h->blk_pmask.p, sizes.p, sizes.p + nb + 1);
    st = cub_call(h, [&](void* tmp, size_t& bytes) {
      return cub::DeviceScan::ExclusiveSum(tmp, bytes, sizes.p, h->blk_voff.p, (int64_t)(nb + 1), s);
    });
    if (st) return st;
    unsigned long long total = 0, pads = 0;
    CK(cudaMemcpyAsync(&total, h->blk_voff.p + nb, sizeof total, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(&pads, sizes.p + nb + 1, sizeof pads, cudaMemcpyDeviceToHost, s));
    CK(h->off_t.reserve(h->nt * kPairs2 + 1, s));
    CK(h->off_b.reserve(h->nbm * kPairs2 + 1, s));
    CK(h->off_p.reserve(h->np * kPairs4 + 1, s));
    k_pair_offsets<<<grid_for(np, 256), 256, 0, s>>>(svals.p, incl.p, np, h->blk_start.p, h->blk_voff.p,
                                                     h->blk_lay.p, h->off_t.p, h->off_b.p, h->off_p.p);
    CK(cudaStreamSynchronize(s));
    sizes.release();
    h->v_words = (size_t)total;
    h->v_pad = (size_t)pads;
  }
  // 6. row-node adjacency in (row node, column node) order: a stable sort of the blocks by their column node
  // J (kb bits) gives every row its blocks (I, r), I <= r, in I order; the block order gives its (r, J), J > r
  size_t nn = h->nodes_number;
  DevBuf<uint32_t> jcol, sjcol, jidx, by_col, alen, aoff;
  CK(jcol.reserve(nb, s));
  CK(sjcol.reserve(nb, s));
  CK(jidx.reserve(nb, s));
  CK(by_col.reserve(nb, s));
  k_block_cols<<<grid_for(nb, 256), 256, 0, s>>>(nb, h->blk_J.p, jcol.p, jidx.p);
  st = cub_call(h, [&](void* tmp, size_t& bytes) {
    return cub::DeviceRadixSort::SortPairs(tmp, bytes, jcol.p, sjcol.p, jidx.p, by_col.p, (int64_t)nb, 0, kb, s);
  });
  if (st) return st;
  DevBuf<int32_t> jf, je, i_f, ie;
  CK(jf.reserve(nn, s));
  CK(je.reserve(nn, s));
  CK(i_f.reserve(nn, s));
  CK(ie.reserve(nn, s));
  CK(cudaMemsetAsync(jf.p, 0xff, nn * sizeof(int32_t), s));
  CK(cudaMemsetAsync(je.p, 0xff, nn * sizeof(int32_t), s));
  CK(cudaMemsetAsync(i_f.p, 0xff, nn * sizeof(int32_t), s));
  CK(cudaMemsetAsync(ie.p, 0xff, nn * sizeof(int32_t), s));
  k_runs<<<grid_for(nb, 256), 256, 0, s>>>(sjcol.p, nb, jf.p, je.p);
  k_runs<<<grid_for(nb, 256), 256, 0, s>>>(h->blk_I.p, nb, i_f.p, ie.p);
  CK(alen.reserve(nn + 1, s));
  CK(aoff.reserve(nn + 1, s));
  k_adj_lens<<<grid_for(nn + 1, 256), 256, 0, s>>>(nn, jf.p, je.p, i_f.p, ie.p, h->blk_J.p, alen.p);
  st = cub_call(h, [&](void* tmp, size_t& bytes) {
    return cub::DeviceScan::ExclusiveSum(tmp, bytes, alen.p, aoff.p, (int64_t)(nn + 1), s);
  });
  if (st) return st;
  const size_t na = 2 * nb;  // at most: every block once in its row, the off-diagonal ones once more
  DevBuf<uint64_t> sakeys;
  DevBuf<uint32_t> savals;
  CK(sakeys.reserve(na, s));
  CK(savals.reserve(na, s));
  DevBuf<int32_t> seg_b, seg_e;
  DevBuf<int64_t> row_nnz, gcount, gbase;
  CK(seg_b.reserve(nn, s));
  CK(seg_e.reserve(nn, s));
  CK(row_nnz.reserve(nrows + 1, s));
  CK(gcount.reserve(nn + 1, s));
  CK(gbase.reserve(nn + 1, s));
  CK(cudaMemsetAsync(row_nnz.p, 0, (nrows + 1) * sizeof(int64_t), s));
  CK(cudaMemsetAsync(gcount.p, 0, (nn + 1) * sizeof(int64_t), s));
  k_adj_fill<<<grid_for(nn, 128), 128, 0, s>>>(nn, jf.p, je.p, i_f.p, ie.p, h->blk_I.p, h->blk_J.p, by_col.p, aoff.p,
                                               kb, sakeys.p, savals.p, seg_b.p, seg_e.p);
  k_row_counts<<<grid_for(nn, 128), 128, 0, s>>>(nn, seg_b.p, seg_e.p, savals.p, h->blk_mask.p, h->blk_maskT.p,
                                                 row_nnz.p, gcount.p);
  st = cub_call(h, [&](void* tmp, size_t& bytes) {
    return cub::DeviceScan::ExclusiveSum(tmp, bytes, row_nnz.p, h->row_ptr.p, (int64_t)(nrows + 1), s);
  });
  if (st) return st;
  st = cub_call(h, [&](void* tmp, size_t& bytes) {
    return cub::DeviceScan::ExclusiveSum(tmp, bytes, gcount.p, gbase.p, (int64_t)(nn + 1), s);
  });
  if (st) return st;
  int64_t nnz = 0, ng = 0;
  CK(cudaMemcpyAsync(&nnz, h->row_ptr.p + nrows, sizeof nnz, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(&ng, gbase.p + nn, sizeof ng, cudaMemcpyDeviceToHost, s));
  // node chunks of the row fill and their first entries
  size_t fill_node[kFillChunks + 1];
  int64_t fill_entry[kFillChunks + 1];
  for (int c = 0; c <= kFillChunks; ++c) {
    fill_node[c] = nn * (size_t)c / kFillChunks;
    fill_entry[c] = 0;
    if (pc && c > 0 && c < kFillChunks)
      CK(cudaMemcpyAsync(&fill_entry[c], h->row_ptr.p + 6 * fill_node[c], sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  }
  CK(cudaStreamSynchronize(s));
  h->nnz = nnz;
  h->n_groups = ng;
  fill_entry[kFillChunks] = nnz;
  const bool early = pc && h->copy_stream && nnz <= pc->capacity;
  CK(h->col_idx.reserve(nnz + 1, s));
  CK(h->values.reserve(nnz + 1, s));
  CK(h->nnz_group.reserve(nnz + 1, s));
  CK(h->src_map.reserve(nnz + 1, s));
  CK(h->g_row.reserve(ng + 1, s));
  CK(h->g_col.reserve(ng + 1, s));
  CK(h->g_kind.reserve(ng + 1, s));
  // block-sum slots by contribution count, their descriptors, then the CSR rows with the source of every entry
  {
    const size_t st_ = nb + 1;
    DevBuf<unsigned long long> sz;
    CK(sz.reserve(kSlotCats * st_, s));
    CK(h->sbase.reserve(kSlotCats * st_, s));
    for (int g = 0; g < kSlotCats; ++g) CK(cudaMemsetAsync(sz.p + g * st_ + nb, 0, sizeof(unsigned long long), s));
    k_slot_sizes<<<grid_for(nb, 256), 256, 0, s>>>(nb, h->blk_count.p, h->blk_pmask.p, h->blk_lay.p, sz.p);
    for (int g = 0; g < kSlotCats; ++g) {
      st = cub_call(h, [&](void* tmp, size_t& bytes) {
        return cub::DeviceScan::ExclusiveSum(tmp, bytes, sz.p + g * st_, h->sbase.p + g * st_, (int64_t)st_, s);
      });
      if (st) return st;
    }
    unsigned long long tot[kSlotCats];
    for (int g = 0; g < kSlotCats; ++g)
      CK(cudaMemcpyAsync(&tot[g], h->sbase.p + g * st_ + nb, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    // descriptor order: 2, 3, 4, 5+ contributions (the S slots), then the check-only ones
    unsigned long long at = 0;
    for (int g = 1; g < kSlotCats; ++g) {
      h->slot_off[g] = at;
      at += tot[g];
    }
    h->s_words = (size_t)at;
    h->slot_off[0] = at;
    h->n_desc = (size_t)(at + tot[0]);
    h->vs_off = ((unsigned long long)h->v_words + 3ull) & ~3ull;  // S 32-byte aligned after the scratch
    if (h->vs_off + h->s_words + 4 >= (1ull << 32))
      return h->fail(FEM_GPU_ERR_ARGUMENT, "model too large: %llu doubles of scratch and sums (limit 2^32)",
                     (unsigned long long)(h->vs_off + h->s_words));
    CK(h->V.reserve(h->vs_off + h->s_words + 4, s));
    SlotLayout L;
    L.base = h->sbase.p;
    L.stride = st_;
    for (int g = 0; g < kSlotCats; ++g) L.off[g] = h->slot_off[g];
    L.vs_off = h->vs_off;
    CK(h->slot_desc.reserve(h->n_desc + 1, s));
    CK(cudaMemsetAsync(h->flag.p + 1, 0, sizeof(int), s));
    if (early) {
      // row_ptr is final: it goes back while the slots and columns are made.  From here on the phase makes no
      // device-to-host read on its own stream (one would queue behind these copies on the copy engine).
      CK(cudaEventRecord(h->copy_ev, s));
      CK(cudaStreamWaitEvent(h->copy_stream, h->copy_ev, 0));
      CK(cudaMemcpyAsync(pc->row_ptr, h->row_ptr.p, (nrows + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost,
                         h->copy_stream));
    }
    k_slot_desc<<<grid_for(nb, 256), 256, 0, s>>>(nb, h->blk_count.p, h->blk_pmask.p, h->blk_lay.p, h->blk_voff.p, L,
                                                  h->slot_desc.p, h->flag.p + 1);
    // the rows in node chunks when the columns go back early (each chunk's columns follow it on the copy
    // stream), else in one launch
    const int chunks = early ? kFillChunks : 1;
    for (int c = 0; c < chunks; ++c) {
      const size_t n0 = early ? fill_node[c] : 0, n1 = early ? fill_node[c + 1] : nn;
      if (n1 > n0)
        k_row_fill<<<grid_for((n1 - n0) * kRowLanes, 256), 256, 0, s>>>(
            n0, n1, seg_b.p, seg_e.p, sakeys.p, kb, savals.p, h->blk_mask.p, h->blk_maskT.p, h->blk_lay.p,
            h->blk_count.p, h->blk_voff.p, L, h->row_ptr.p, gbase.p, h->col_idx.p, h->nnz_group.p, h->src_map.p,
            h->g_row.p, h->g_col.p, h->g_kind.p, (unsigned long long)nnz, (unsigned long long)ng,
            h->vs_off + h->s_words);
      if (early && fill_entry[c + 1] > fill_entry[c]) {
        if (!h->fill_ev[c]) CK(cudaEventCreateWithFlags(&h->fill_ev[c], cudaEventDisableTiming));
        CK(cudaEventRecord(h->fill_ev[c], s));
        CK(cudaStreamWaitEvent(h->copy_stream, h->fill_ev[c], 0));
        CK(cudaMemcpyAsync(pc->col_idx + fill_entry[c], h->col_idx.p + fill_entry[c],
                           (size_t)(fill_entry[c + 1] - fill_entry[c]) * sizeof(int32_t), cudaMemcpyDeviceToHost,
                           h->copy_stream));
      }
    }
    CK(cudaGetLastError());
    if (early) {
      pc->issued = true;  // the caller reads flag[1] (a node pair shared by 2^24 or more elements) after its pass
    } else {
      int too_many = 0;
      CK(cudaMemcpyAsync(&too_many, h->flag.p + 1, sizeof too_many, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      if (too_many) return h->fail(FEM_GPU_ERR_ARGUMENT, kTooManyMsg);
    }
    sz.release();
  }
  if (!early) CK(cudaStreamSynchronize(s));
  // temporaries
  keys.release();
  skeys.release();
  vals.release();
  svals.release();
  smask.release();
  head.release();
  incl.release();
  jcol.release();
  sjcol.release();
  jidx.release();
  by_col.release();
  alen.release();
  aoff.release();
  jf.release();
  je.release();
  i_f.release();
  ie.release();
  sakeys.release();
  savals.release();
  seg_b.release();
  seg_e.release();
  row_nnz.release();
  gcount.release();
  gbase.release();
  h->pattern_valid = true;
  return FEM_GPU_OK;
}

}  // namespace

extern "C" int fem_gpu_assemble(fem_gpu_t* h) {
  int st = ensure_ready(h);
  if (st) return st;
  for (int attempt = 0; attempt < 2; ++attempt) {
    if (!h->pattern_valid) {
      st = symbolic(h);
      if (st) return st;
    }
    st = numeric_launch(h);
    if (st) return st;
    int flag = 0;
    CK(cudaMemcpyAsync(&flag, h->flag.p, sizeof flag, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaEventElapsedTime(&h->t_elem_ms, h->ev[0], h->ev[1]));
    CK(cudaEventElapsedTime(&h->t_reduce_ms, h->ev[1], h->ev[2]));
    if (!flag) return FEM_GPU_OK;
    h->pattern_valid = false;  // a coordinate/property update changed the exact-zero pattern
  }
  return h->fail(FEM_GPU_ERR_PATTERN_CHANGED, "pattern changed twice in one assemble");
}

extern "C" int fem_gpu_assemble_to_host(fem_gpu_t* h, int64_t* row_ptr, int32_t* col_idx, double* values,
                                        int64_t nnz_capacity, int64_t* nnz) {
  if (!h || !row_ptr || (nnz_capacity > 0 && (!col_idx || !values))) return FEM_GPU_ERR_ARGUMENT;
  int st = ensure_ready(h);
  if (st) return st;
  if (!h->copy_stream) {
    CK(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&h->copy_ev, cudaEventDisableTiming));
  }
  // no copy into the caller's buffers outlives the call, whichever way it returns
  struct DrainOnReturn {
    cudaStream_t s;
    ~DrainOnReturn() { cudaStreamSynchronize(s); }
  } drain_on_return{h->copy_stream};
  const size_t nrows = (size_t)h->nodes_number * 6;
  for (int attempt = 0; attempt < 2; ++attempt) {
    PatternCopy pc{row_ptr, col_idx, nnz_capacity};
    if (!h->pattern_valid) {
      st = symbolic(h, &pc);
      if (st) return st;
    }
    if (nnz) *nnz = h->nnz;
    if (h->nnz > nnz_capacity)
      return h->fail(FEM_GPU_ERR_ARGUMENT, "the CSR has %lld entries, the buffers room for %lld",
                     (long long)h->nnz, (long long)nnz_capacity);
    if (!pc.issued) {
      // the pattern goes back on the copy stream while the numeric pass runs (it writes only the values)
      CK(cudaEventRecord(h->copy_ev, h->stream));
      CK(cudaStreamWaitEvent(h->copy_stream, h->copy_ev, 0));
    }
    st = numeric_launch(h);
    if (st) return st;
    if (!pc.issued) {
      CK(cudaMemcpyAsync(row_ptr, h->row_ptr.p, (nrows + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost,
                         h->copy_stream));
      if (h->nnz)
        CK(cudaMemcpyAsync(col_idx, h->col_idx.p, (size_t)h->nnz * sizeof(int32_t), cudaMemcpyDeviceToHost,
                           h->copy_stream));
    }
    int flag[2] = {0, 0};
    CK(cudaMemcpyAsync(flag, h->flag.p, (pc.issued ? 2 : 1) * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    if (h->nnz)
      CK(cudaMemcpyAsync(values, h->values.p, (size_t)h->nnz * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaStreamSynchronize(h->copy_stream));
    if (flag[1]) {
      h->pattern_valid = false;
      return h->fail(FEM_GPU_ERR_ARGUMENT, kTooManyMsg);
    }
    CK(cudaEventElapsedTime(&h->t_elem_ms, h->ev[0], h->ev[1]));
    CK(cudaEventElapsedTime(&h->t_reduce_ms, h->ev[1], h->ev[2]));
    if (!flag[0]) return FEM_GPU_OK;
    h->pattern_valid = false;  // a coordinate/property update changed the exact-zero pattern
  }
  return h->fail(FEM_GPU_ERR_PATTERN_CHANGED, "pattern changed twice in one assemble");
}

extern "C" int fem_gpu_assemble_numeric_async(fem_gpu_t* h) {
  if (!h) return FEM_GPU_ERR_ARGUMENT;
  if (!h->pattern_valid) return h->fail(FEM_GPU_ERR_STATE, "no valid pattern: call fem_gpu_assemble first");
  return numeric_launch(h);
}

extern "C" int fem_gpu_debug_check(int* checked, int* site, int64_t* index, int64_t* bound) {
#ifdef FEM_GPU_DEBUG
  if (checked) *checked = 1;
#else
  if (checked) *checked = 0;
#endif
  DebugRecord r = {};
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpyFromSymbol(&r, g_dbg, sizeof r);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return FEM_GPU_ERR_CUDA;
  }
  if (site) *site = r.flag ? r.site : 0;
  if (index) *index = (int64_t)r.index;
  if (bound) *bound = (int64_t)r.bound;
  if (r.flag) {
    const DebugRecord zero = {};
    e = cudaMemcpyToSymbol(g_dbg, &zero, sizeof zero);
    if (e != cudaSuccess) return FEM_GPU_ERR_CUDA;
  }
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_check_pattern(fem_gpu_t* h) {
  if (!h || !h->stream) return FEM_GPU_ERR_ARGUMENT;
  int flag = 0;
  CK(cudaMemcpyAsync(&flag, h->flag.p, sizeof flag, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (flag) {
    h->pattern_valid = false;
    return h->fail(FEM_GPU_ERR_PATTERN_CHANGED, "the exact-zero pattern changed; call fem_gpu_assemble");
  }
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_set_node_coordinates(fem_gpu_t* h, const double* xyz, size_t n_nodes) {
  if (!h || !xyz || n_nodes != h->n_nodes) return FEM_GPU_ERR_ARGUMENT;
  int st = ensure_ready(h);
  if (st) return st;
  std::vector<double> a(n_nodes), b(n_nodes), c(n_nodes);
  for (size_t i = 0; i < n_nodes; ++i) {
    a[i] = xyz[3 * i];
    b[i] = xyz[3 * i + 1];
    c[i] = xyz[3 * i + 2];
  }
  CK(cudaMemcpyAsync(h->dx.p, a.data(), n_nodes * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->dy.p, b.data(), n_nodes * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->dz.p, c.data(), n_nodes * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  // later duplicate checks compare against the nodes' new coordinates
  for (size_t i = 0; i < n_nodes; ++i) h->node_ck[i] = coord_key(a[i], b[i], c[i]);
  h->node_coords = PartTable();
  h->coords_built = 0;
  h->numeric_done = false;
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_set_plate_properties(fem_gpu_t* h, const double* young, const double* poisson,
                                            const double* thickness, const double* shear_factor, size_t n) {
  if (!h || n != h->np || !young || !poisson || !thickness || !shear_factor) return FEM_GPU_ERR_ARGUMENT;
  CK(cudaMemcpyAsync(h->p_E.p, young, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->p_nu.p, poisson, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->p_t.p, thickness, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->p_ks.p, shear_factor, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  h->numeric_done = false;
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_get_csr_sizes(fem_gpu_t* h, int64_t* n_rows, int64_t* nnz) {
  if (!h) return FEM_GPU_ERR_ARGUMENT;
  if (!h->numeric_done || !h->pattern_valid) return h->fail(FEM_GPU_ERR_STATE, "call fem_gpu_assemble first");
  if (n_rows) *n_rows = (int64_t)h->nodes_number * 6;
  if (nnz) *nnz = h->nnz;
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_get_csr(fem_gpu_t* h, int64_t* row_ptr, int32_t* col_idx, double* values) {
  int st = fem_gpu_get_csr_sizes(h, nullptr, nullptr);
  if (st) return st;
  size_t nrows = (size_t)h->nodes_number * 6;
  if (row_ptr) CK(cudaMemcpyAsync(row_ptr, h->row_ptr.p, (nrows + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, h->stream));
  if (col_idx && h->nnz)
    CK(cudaMemcpyAsync(col_idx, h->col_idx.p, h->nnz * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
  if (values && h->nnz)
    CK(cudaMemcpyAsync(values, h->values.p, h->nnz * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_get_csr_values(fem_gpu_t* h, double* values) { return fem_gpu_get_csr(h, nullptr, nullptr, values); }

extern "C" int fem_gpu_get_csr_device(fem_gpu_t* h, const int64_t** row_ptr, const int32_t** col_idx,
                                      const double** values) {
  int st = fem_gpu_get_csr_sizes(h, nullptr, nullptr);
  if (st) return st;
  if (row_ptr) *row_ptr = h->row_ptr.p;
  if (col_idx) *col_idx = h->col_idx.p;
  if (values) *values = h->values.p;
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_get_node_count(fem_gpu_t* h, int64_t* n_nodes) {
  if (!h || !n_nodes) return FEM_GPU_ERR_ARGUMENT;
  *n_nodes = (int64_t)h->n_nodes;
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_get_index_node_numbers(fem_gpu_t* h, uint32_t* numbers) {
  if (!h || (!numbers && h->n_nodes)) return FEM_GPU_ERR_ARGUMENT;
  if (h->n_nodes) memcpy(numbers, h->idx_number.data(), h->n_nodes * sizeof(uint32_t));
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_get_group_count(fem_gpu_t* h, int64_t* n_groups) {
  if (!h || !n_groups) return FEM_GPU_ERR_ARGUMENT;
  if (!h->pattern_valid) return h->fail(FEM_GPU_ERR_STATE, "call fem_gpu_assemble first");
  *n_groups = h->n_groups;
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_get_groups(fem_gpu_t* h, int32_t* row_node, int32_t* col_node, uint8_t* kind,
                                  int32_t* nnz_group) {
  if (!h) return FEM_GPU_ERR_ARGUMENT;
  if (!h->pattern_valid) return h->fail(FEM_GPU_ERR_STATE, "call fem_gpu_assemble first");
  size_t ng = (size_t)h->n_groups, nz = (size_t)h->nnz;
  if (row_node && ng) CK(cudaMemcpyAsync(row_node, h->g_row.p, ng * 4, cudaMemcpyDeviceToHost, h->stream));
  if (col_node && ng) CK(cudaMemcpyAsync(col_node, h->g_col.p, ng * 4, cudaMemcpyDeviceToHost, h->stream));
  if (kind && ng) CK(cudaMemcpyAsync(kind, h->g_kind.p, ng, cudaMemcpyDeviceToHost, h->stream));
  if (nnz_group && nz) CK(cudaMemcpyAsync(nnz_group, h->nnz_group.p, nz * 4, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return FEM_GPU_OK;
}

namespace {
int rotation_of(fem_gpu* h, int kind, uint32_t number, double* r9) {
  if (!h || !r9) return FEM_GPU_ERR_ARGUMENT;
  const NumberMap& m = kind == kTruss ? h->t_by_num : kind == kBeam ? h->b_by_num : h->p_by_num;
  const int64_t found = m.find(number);
  const char* nm = kind == kTruss ? "Truss" : kind == kBeam ? "Beam" : "Plate";
  if (found < 0) return h->fail(FEM_GPU_ERR_ARGUMENT, "%s element with number %u does not exist!", nm, number);
  DevBuf<double> out;
  CK(out.reserve(9, h->stream));
  if (kind == kTruss)
    k_rotation<<<1, 1, 0, h->stream>>>(kind, h->nodes(), h->t_n1.p, h->t_n2.p, nullptr, nullptr, h->beams(), h->rel_tol,
                                       h->abs_tol, (size_t)found, out.p);
  else if (kind == kBeam)
    k_rotation<<<1, 1, 0, h->stream>>>(kind, h->nodes(), nullptr, nullptr, nullptr, nullptr, h->beams(), h->rel_tol,
                                       h->abs_tol, (size_t)found, out.p);
  else
    k_rotation<<<1, 1, 0, h->stream>>>(kind, h->nodes(), h->p_n1.p, h->p_n2.p, h->p_n3.p, h->p_n4.p, h->beams(),
                                       h->rel_tol, h->abs_tol, (size_t)found, out.p);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(r9, out.p, 9 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  out.release();
  return FEM_GPU_OK;
}
}  // namespace

extern "C" int fem_gpu_get_truss_rotation(fem_gpu_t* h, uint32_t number, double* r9) {
  return rotation_of(h, kTruss, number, r9);
}
extern "C" int fem_gpu_get_beam_rotation(fem_gpu_t* h, uint32_t number, double* r9) {
  return rotation_of(h, kBeam, number, r9);
}
extern "C" int fem_gpu_get_plate_rotation(fem_gpu_t* h, uint32_t number, double* r9) {
  return rotation_of(h, kPlate, number, r9);
}

extern "C" int fem_gpu_get_element_counts(fem_gpu_t* h, int64_t* n_truss, int64_t* n_beam, int64_t* n_plate) {
  if (!h) return FEM_GPU_ERR_ARGUMENT;
  if (n_truss) *n_truss = (int64_t)h->nt;
  if (n_beam) *n_beam = (int64_t)h->nbm;
  if (n_plate) *n_plate = (int64_t)h->np;
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_get_stream(fem_gpu_t* h, void** stream) {
  if (!h || !stream) return FEM_GPU_ERR_ARGUMENT;
  int st = ensure_ready(h);
  if (st) return st;
  *stream = (void*)h->stream;
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_numeric_launch_count(fem_gpu_t* h, int* n_launches) {
  if (!h || !n_launches) return FEM_GPU_ERR_ARGUMENT;
  *n_launches = (h->nt ? 1 : 0) + (h->nbm ? 1 : 0) + (h->np ? 1 : 0) + (h->n_blocks ? 2 : 0);
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_get_pattern_stats(fem_gpu_t* h, int64_t* n_blocks, int64_t* n_contributions,
                                         int64_t* scratch_doubles, int64_t* sum_slots) {
  if (!h) return FEM_GPU_ERR_ARGUMENT;
  if (!h->pattern_valid) return h->fail(FEM_GPU_ERR_STATE, "call fem_gpu_assemble first");
  if (n_blocks) *n_blocks = (int64_t)h->n_blocks;
  if (n_contributions) *n_contributions = (int64_t)h->n_pairs;
  if (scratch_doubles) *scratch_doubles = (int64_t)(h->v_words - h->v_pad);
  if (sum_slots) *sum_slots = (int64_t)h->s_words;
  return FEM_GPU_OK;
}

extern "C" int fem_gpu_last_numeric_timing(fem_gpu_t* h, float* element_ms, float* reduce_ms) {
  if (!h) return FEM_GPU_ERR_ARGUMENT;
  if (!h->numeric_done) return h->fail(FEM_GPU_ERR_STATE, "no numeric pass yet");
  CK(cudaEventSynchronize(h->ev[2]));
  CK(cudaEventElapsedTime(&h->t_elem_ms, h->ev[0], h->ev[1]));
  CK(cudaEventElapsedTime(&h->t_reduce_ms, h->ev[1], h->ev[2]));
  if (element_ms) *element_ms = h->t_elem_ms;
  if (reduce_ms) *reduce_ms = h->t_reduce_ms;
  return FEM_GPU_OK;
}

// batched assembly of many structures (reuses the kernels and the handle above)
#include "fem_batch.cuh"
// batches built from the host arrays of many structures (one union model)
#include "fem_batch_arrays.cuh"
// vector-Jacobian product (reuses the element arithmetic and the handle above)
#include "fem_adjoint.cuh"
// sparse separation of the assembled stiffness by the imposed displacements
#include "fem_separate.cuh"
// concentrated, line and surface loads and the forces vector
#include "fem_loads.cuh"
// PCG solution of the separated system and the reactions
#include "fem_solve.cuh"
#include "fem_results.cuh"
