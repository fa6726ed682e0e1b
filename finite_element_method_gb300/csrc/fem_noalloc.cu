// fem_noalloc.cu -- fem_gpu_assemble_dense_noalloc: dense assembly of one small
// structure into caller-provided device memory, with no device allocation.
//
// Some callers cannot call cudaMalloc: code that owns every byte of device
// memory through its own arena or pool (a host runtime that hands out
// pre-sized buffers and forbids allocations behind its back), code running
// where an allocation could stall or fail unpredictably (a solver inner loop
// with a fixed memory budget), and code that must not change the process's
// memory footprint once it is set up.  This entry point takes device pointers
// for every input and for the output and keeps its working memory in one
// file-scope __device__ array of fixed size, so it never allocates.
//
// The working array is sized for kNoallocMaxPairs = 32768 node-pair blocks
// (3 per truss or beam, 10 per plate: at most 3276 plates or 10922 two-node
// elements per call); it takes about 10 MB on every GPU where the library's
// device code is loaded, until the process exits.  Under CUDA's default lazy
// module loading that happens when the library's kernels are first used on a
// device, not when the library is opened.  Its device address is looked up
// once per device, on the first call made with that device current; make that
// first call before any stream capture.
// All calls on a device share it, and it keeps the last call's contents:
// calls that overlap on the GPU (different streams, or threads calling at the
// same time) race on it and must be serialised by the caller.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "../../include/fem_gpu.h"
#include "element_math.cuh"

using namespace femgpu;

namespace {

constexpr size_t kNoallocMaxPairs = 32768;          // a power of two (the sort below relies on it)
constexpr int kPairBits = 15;                         // bits of a block index below kNoallocMaxPairs
constexpr uint32_t kNoallocMaxNodes = 1u << 24;       // node indices fit 24 bits of a sort key
// layout of the working array, in 8-byte words:
//   [0, 36 P)          element node-pair blocks (36 doubles each), element order
//   [36 P, 37 P)       node-pair key (lo << 32 | hi) per block
//   [37 P, 38 P)       sort keys (lo << 39 | hi << 15 | block), sorted in place
//   [38 P, 38.5 P)     next block with the same key (int32), -1 = none
//   [38.5 P, 39 P)     1 if the block is the first of its key (int32)
//   [39 P]             error flag
constexpr size_t kWordsV = 36 * kNoallocMaxPairs;
constexpr size_t kWordsKey = kNoallocMaxPairs;
constexpr size_t kWordsSort = kNoallocMaxPairs;
constexpr size_t kWordsLinks = kNoallocMaxPairs;  // next + head, two int32 per word
constexpr size_t kNoallocWords = kWordsV + kWordsKey + kWordsSort + kWordsLinks + 1;

static __device__ __align__(256) unsigned long long g_noalloc_scratch[kNoallocWords];

struct Scratch {
  double* V;
  unsigned long long* key;
  unsigned long long* sort;
  int32_t* next;
  int32_t* head;
  int* flag;
};

__host__ __device__ inline Scratch carve(unsigned long long* base) {
  Scratch s;
  s.V = reinterpret_cast<double*>(base);
  s.key = base + kWordsV;
  s.sort = base + kWordsV + kWordsKey;
  int32_t* links = reinterpret_cast<int32_t*>(base + kWordsV + kWordsKey + kWordsSort);
  s.next = links;
  s.head = links + kNoallocMaxPairs;
  s.flag = reinterpret_cast<int*>(base + kWordsV + kWordsKey + kWordsSort + kWordsLinks);
  return s;
}

__device__ __forceinline__ void get_node(const double* xyz, int32_t i, double o[3]) {
  o[0] = xyz[3 * (size_t)i];
  o[1] = xyz[3 * (size_t)i + 1];
  o[2] = xyz[3 * (size_t)i + 2];
}

// store a 6x6 block in (lo, hi) orientation: transposed when the element's
// first node of the pair has the larger index
__device__ __forceinline__ void put_block(Scratch s, size_t q, int32_t I, int32_t J, const double blk[36]) {
  bool tr = I > J;
  double* dst = s.V + q * 36;
#pragma unroll
  for (int a = 0; a < 6; ++a)
#pragma unroll
    for (int b = 0; b < 6; ++b) dst[6 * a + b] = tr ? blk[6 * b + a] : blk[6 * a + b];
  uint32_t lo = (uint32_t)(I < J ? I : J), hi = (uint32_t)(I < J ? J : I);
  s.key[q] = ((unsigned long long)lo << 32) | hi;
}

__device__ __forceinline__ bool bad_node(int32_t i, uint32_t n_nodes) { return i < 0 || (uint32_t)i >= n_nodes; }

// trusses: props per element E, A, A2 (NaN = none); pairs (1,1), (1,2), (2,2)
__global__ void k_na_truss(Scratch s, const double* __restrict__ xyz, uint32_t n_nodes, const int32_t* __restrict__ nd,
                           const double* __restrict__ pr, size_t n, size_t q0, double abs_tol) {
  size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= n) return;
  int32_t I = nd[2 * e], J = nd[2 * e + 1];
  double blk[36];
#pragma unroll
  for (int k = 0; k < 36; ++k) blk[k] = 0.0;
  double g[9];
  bool ok = !bad_node(I, n_nodes) && !bad_node(J, n_nodes);
  if (ok) {
    double x1[3], x2[3];
    get_node(xyz, I, x1);
    get_node(xyz, J, x2);
    ok = truss_block(x1, x2, pr[3 * e], pr[3 * e + 1], pr[3 * e + 2], abs_tol, g);
  }
  if (!ok) {
    atomicOr(s.flag, 1);
    I = J = 0;
#pragma unroll
    for (int k = 0; k < 9; ++k) g[k] = 0.0;
  }
#pragma unroll
  for (int p = 0; p < 3; ++p) {
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) blk[6 * a + b] = p == 1 ? -g[3 * a + b] : g[3 * a + b];
    int32_t A = p == 2 ? J : I, B = p == 0 ? I : J;
    put_block(s, q0 + 3 * e + p, A, B, blk);
  }
}

// beams: props per element E, nu, A, I11, I22, I12, It, k, axis x, y, z
__global__ void k_na_beam(Scratch s, const double* __restrict__ xyz, uint32_t n_nodes, const int32_t* __restrict__ nd,
                          const double* __restrict__ pr, size_t n, size_t q0, double rel_tol, double abs_tol) {
  size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= n) return;
  int32_t I = nd[2 * e], J = nd[2 * e + 1];
  const double* p = pr + 11 * e;
  BeamBlocks B;
  bool ok = !bad_node(I, n_nodes) && !bad_node(J, n_nodes);
  if (ok) {
    double x1[3], x2[3], axis[3] = {p[8], p[9], p[10]};
    get_node(xyz, I, x1);
    get_node(xyz, J, x2);
    ok = beam_blocks(x1, x2, p[0], p[1], p[2], p[3], p[4], p[5], p[6], p[7], axis, rel_tol, abs_tol, B);
  }
  if (!ok) {
    atomicOr(s.flag, 1);
    I = J = 0;
#pragma unroll
    for (int k = 0; k < 9; ++k) B.uu[k] = B.ut[k] = B.th[k] = B.tu[k] = B.thth2[k] = 0.0;
  }
  double blk[36];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      blk[6 * a + c] = B.uu[3 * a + c];
      blk[6 * a + 3 + c] = B.ut[3 * a + c];
      blk[6 * (3 + a) + c] = B.ut[3 * c + a];
      blk[6 * (3 + a) + 3 + c] = B.th[3 * a + c];
    }
  put_block(s, q0 + 3 * e + 0, I, I, blk);
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      blk[6 * a + c] = -B.uu[3 * a + c];
      blk[6 * a + 3 + c] = B.ut[3 * a + c];
      blk[6 * (3 + a) + c] = B.tu[3 * a + c];
      blk[6 * (3 + a) + 3 + c] = B.thth2[3 * a + c];
    }
  put_block(s, q0 + 3 * e + 1, I, J, blk);
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      blk[6 * a + c] = B.uu[3 * a + c];
      blk[6 * a + 3 + c] = -B.ut[3 * a + c];
      blk[6 * (3 + a) + c] = -B.ut[3 * c + a];
      blk[6 * (3 + a) + 3 + c] = B.th[3 * a + c];
    }
  put_block(s, q0 + 3 * e + 2, J, J, blk);
}

// plates: props per element E, nu, t, k; pairs (i, j), i <= j, of the 4 nodes
__global__ void k_na_plate(Scratch s, const double* __restrict__ xyz, uint32_t n_nodes, const int32_t* __restrict__ nd,
                           const double* __restrict__ pr, size_t n, size_t q0, double abs_tol) {
  size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= n) return;
  int32_t nidx[4] = {nd[4 * e], nd[4 * e + 1], nd[4 * e + 2], nd[4 * e + 3]};
  bool ok = true;
#pragma unroll
  for (int k = 0; k < 4; ++k) ok = ok && !bad_node(nidx[k], n_nodes);
  // a node used twice would make two of the element's node pairs one block
  // (the handle path rejects such plates: their nodes lie on a line)
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int l = k + 1; l < 4; ++l) ok = ok && nidx[k] != nidx[l];
  double X[4][3];
  double R[9];
  set_identity(R);
  if (ok) {
#pragma unroll
    for (int k = 0; k < 4; ++k) get_node(xyz, nidx[k], X[k]);
    // the geometry checks of the handle path (structs/plate.rs:58-158): nodes on a line,
    // not on one plane, not convex
    bool hull_ok = false;
    ok = !quad_on_line(X[0], X[1], X[2], X[3]) && quad_on_plane(X[0], X[1], X[2], X[3], abs_tol) &&
         quad_hull_size(X[0], X[1], X[2], X[3], abs_tol, hull_ok) == 4 && hull_ok;
    if (ok) ok = plate_rotation(X[1], X[2], X[3], abs_tol, R);
  }
  if (!ok) {
    atomicOr(s.flag, 1);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      nidx[k] = 0;
      X[k][0] = k == 0 || k == 3 ? 1.0 : 0.0;
      X[k][1] = k < 2 ? 1.0 : 0.0;
      X[k][2] = 0.0;
    }
    set_identity(R);
  }
  const bool ident = is_identity(R);
  double xl[4], yl[4];
  plate_local_xy(X, R, ident, xl, yl);
  const double* p = pr + 4 * e;
  PlateCore C;
  plate_core(xl, yl, p[0], p[1], p[2], p[3], C);
  const int PI[10] = {0, 0, 0, 0, 1, 1, 1, 2, 2, 3};
  const int PJ[10] = {0, 1, 2, 3, 1, 2, 3, 2, 3, 3};
#pragma unroll 1
  for (int q = 0; q < 10; ++q) {
    int i = PI[q], j = PJ[q];
    double blk[36];
    plate_local_block(C, i, j, blk);
    if (!ident) {
      double o[36];
      plate_rotate_block(R, i == j, blk, o);
#pragma unroll
      for (int k = 0; k < 36; ++k) blk[k] = o[k];
    }
    if (!ok) {
#pragma unroll
      for (int k = 0; k < 36; ++k) blk[k] = 0.0;
    }
    put_block(s, q0 + 10 * e + q, nidx[i], nidx[j], blk);
  }
}

// sort keys: the block's node pair above its index, so that sorting them puts
// the blocks of one node pair together in element order; padding sorts last
__global__ void k_na_sort_keys(Scratch s, size_t P, size_t P2) {
  size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (q >= P2) return;
  if (q >= P) {
    s.sort[q] = ~0ull;
    return;
  }
  const unsigned long long k = s.key[q];
  const unsigned long long lo = k >> 32, hi = k & 0xffffffffull;
  s.sort[q] = (lo << (24 + kPairBits)) | (hi << kPairBits) | (unsigned long long)q;
}

// bitonic sort of the P2 (a power of two, <= kNoallocMaxPairs) sort keys by
// one block of threads; the keys are distinct (they hold the block index)
__global__ void __launch_bounds__(1024) k_na_sort(Scratch s, size_t P2) {
  unsigned long long* a = s.sort;
  for (size_t k = 2; k <= P2; k <<= 1)
    for (size_t j = k >> 1; j > 0; j >>= 1) {
      for (size_t i = threadIdx.x; i < P2; i += blockDim.x) {
        const size_t l = i ^ j;
        if (l > i) {
          const unsigned long long x = a[i], y = a[l];
          if ((x > y) == ((i & k) == 0)) {
            a[i] = y;
            a[l] = x;
          }
        }
      }
      __syncthreads();
    }
}

// next[q]: the following block with the same key; head[q]: q is its key's first block
__global__ void k_na_links(Scratch s, size_t P) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= P) return;
  const unsigned long long mask = (1ull << kPairBits) - 1ull;
  const unsigned long long v = s.sort[i];
  const int32_t q = (int32_t)(v & mask);
  const unsigned long long k = v >> kPairBits;
  s.head[q] = (i == 0 || (s.sort[i - 1] >> kPairBits) != k) ? 1 : 0;
  s.next[q] = (i + 1 < P && (s.sort[i + 1] >> kPairBits) == k) ? (int32_t)(s.sort[i + 1] & mask) : -1;
}

__global__ void k_na_zero(double* K, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) K[i] = 0.0;
}

// one thread per (head block, entry): sum the key's blocks in element order and
// store the entry and its mirror in the dense matrix
__global__ void k_na_sum(Scratch s, size_t P, size_t n_dof, double* K) {
  size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= P * 36) return;
  size_t q = t / 36;
  int en = (int)(t - 36 * q);
  if (!s.head[q]) return;
  double sum = s.V[q * 36 + en];
  for (int32_t r = s.next[q]; r >= 0; r = s.next[r]) sum = sum + s.V[(size_t)r * 36 + en];
  if (sum == 0.0) sum = 0.0;  // an entry that received nothing but zeros reads +0.0
  unsigned long long k = s.key[q];
  size_t lo = (size_t)(k >> 32), hi = (size_t)(k & 0xffffffffull);
  int a = en / 6, c = en % 6;
  K[(6 * lo + a) * n_dof + 6 * hi + c] = sum;
  if (lo != hi) K[(6 * hi + c) * n_dof + 6 * lo + a] = sum;
}

std::mutex g_mu;
unsigned long long* g_scratch_ptr[64] = {nullptr};

// the device address of the working array on the current device (looked up once per device)
cudaError_t scratch_address(unsigned long long** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = static_cast<unsigned long long*>(p);
  }
  *out = g_scratch_ptr[dev];
  return cudaSuccess;
}

unsigned grid_of(size_t n, unsigned b) { return (unsigned)((n + b - 1) / b); }

}  // namespace

extern "C" int fem_gpu_assemble_dense_noalloc(uint32_t n_nodes, const double* xyz, size_t n_truss,
                                              const int32_t* truss_nodes, const double* truss_props, size_t n_beam,
                                              const int32_t* beam_nodes, const double* beam_props, size_t n_plate,
                                              const int32_t* plate_nodes, const double* plate_props, double rel_tol,
                                              double abs_tol, double* K, void* stream) {
  if (n_nodes == 0 || !xyz || !K || (n_truss && (!truss_nodes || !truss_props)) ||
      (n_beam && (!beam_nodes || !beam_props)) || (n_plate && (!plate_nodes || !plate_props)))
    return FEM_GPU_ERR_ARGUMENT;
  // node indices must fit the sort keys; this also keeps (6 n_nodes)^2 doubles far inside size_t
  if (n_nodes >= kNoallocMaxNodes) return FEM_GPU_ERR_ARGUMENT;
  if (n_truss > kNoallocMaxPairs || n_beam > kNoallocMaxPairs || n_plate > kNoallocMaxPairs)
    return FEM_GPU_ERR_NOALLOC_LIMIT;
  size_t P = 3 * n_truss + 3 * n_beam + 10 * n_plate;
  if (P > kNoallocMaxPairs) return FEM_GPU_ERR_NOALLOC_LIMIT;
  unsigned long long* base = nullptr;
  if (scratch_address(&base) != cudaSuccess) return FEM_GPU_ERR_CUDA;
  Scratch s = carve(base);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  size_t n_dof = (size_t)6 * n_nodes;
  (void)cudaGetLastError();  // a launch error reported below is one of this call's
  if (cudaMemsetAsync(s.flag, 0, sizeof(int), st) != cudaSuccess) return FEM_GPU_ERR_CUDA;
  k_na_zero<<<1024, 256, 0, st>>>(K, n_dof * n_dof);
  if (n_truss) k_na_truss<<<grid_of(n_truss, 128), 128, 0, st>>>(s, xyz, n_nodes, truss_nodes, truss_props, n_truss, 0, abs_tol);
  if (n_beam)
    k_na_beam<<<grid_of(n_beam, 128), 128, 0, st>>>(s, xyz, n_nodes, beam_nodes, beam_props, n_beam, 3 * n_truss,
                                                    rel_tol, abs_tol);
  if (n_plate)
    k_na_plate<<<grid_of(n_plate, 128), 128, 0, st>>>(s, xyz, n_nodes, plate_nodes, plate_props, n_plate,
                                                      3 * n_truss + 3 * n_beam, abs_tol);
  if (P) {
    size_t P2 = 1;
    while (P2 < P) P2 <<= 1;
    k_na_sort_keys<<<grid_of(P2, 256), 256, 0, st>>>(s, P, P2);
    k_na_sort<<<1, 1024, 0, st>>>(s, P2);
    k_na_links<<<grid_of(P, 256), 256, 0, st>>>(s, P);
    k_na_sum<<<grid_of(P * 36, 288), 288, 0, st>>>(s, P, n_dof, K);
  }
  if (cudaGetLastError() != cudaSuccess) return FEM_GPU_ERR_CUDA;
  int flag = 0;
  if (cudaMemcpyAsync(&flag, s.flag, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) return FEM_GPU_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return FEM_GPU_ERR_CUDA;
  return flag ? FEM_GPU_ERR_ARGUMENT : FEM_GPU_OK;
}
