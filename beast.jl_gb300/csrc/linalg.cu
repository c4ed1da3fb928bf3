// linalg.cu -- dense complex LU with partial pivoting, triangular solves, FP64 matvec.
//
// Replaces LAPACK zgetrf/zgetrs behind `\` (src/solvers/lusolver.jl:30, src/solvers/lu.jl:40-47)
// for a device-resident matrix.  Right-looking blocked LU:
//   k_panel    cooperative kernel over the column panel: per column a grid-wide pivot
//              search (max |re|+|im|, first index on ties -- the izamax rule), the row swap
//              and the rank-1 update, with bounded-spin grid barriers (a barrier that gives
//              up sets a status word and the kernel returns; nothing hangs)
//   k_laswp    the panel's row interchanges applied to the other columns
//   k_trsm_tile   U12 = L11^{-1} A12 and (unpivoted path, after k_getrf64 on the diagonal
//                 block) L21 = A21 U11^{-1}
//   k_lu_inv64 + k_panel_apply   the unpivoted c64 panel: diagonal block LU with the
//                 inverses of its triangles, then both triangular solves as products
//   k_gemm     A22 -= L21 U12 (complex, tiled through shared memory)
// The element type is complex FP64 (c128) or complex FP32 (c64).
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "fsplit.h"
#include "internal.h"

// the pivot allocation of a factorisation: ipiv[n], perm[n], then (256-byte aligned) the
// inverses of the 64 x 64 diagonal blocks of L and U
size_t lu_aux_bytes(int64_t n, int dtype) {
  size_t head = ((size_t)2 * n * sizeof(int) + 255) & ~(size_t)255;
  size_t el = dtype == BEAST_C64 ? 8 : 16;
  return head + (size_t)((n + 63) / 64) * 2 * 4096 * el;
}
void* lu_dinv(const int* ipiv, int64_t n) {
  size_t head = ((size_t)2 * n * sizeof(int) + 255) & ~(size_t)255;
  return (void*)(reinterpret_cast<const char*>(ipiv) + head);
}

bool tc_gemm_supported(const void* A, int64_t lda, int K);
size_t tc_gemm_work_bytes(int64_t M, int64_t N, int K);
int tc_gemm_sub(beast_ctx* ctx, float2* Mat, int64_t lda, int64_t rowA, int64_t colA, int64_t colB,
                int64_t M0, int64_t N0, int64_t M1, int64_t N1, int K, void* work, size_t work_bytes,
                bool prepped);
int tc_gemm_sym(beast_ctx* ctx, float2* Mat, int64_t lda, int64_t rowA, int64_t colA, int64_t rowB, int64_t M0,
                int64_t N0, int K, bool lower, void* work, size_t work_bytes, bool prepped, int64_t a_skip = 0);

namespace {

template <typename R>
struct CT;
template <>
struct CT<double> {
  typedef double2 T;
};
template <>
struct CT<float> {
  typedef float2 T;
};

template <typename T>
__device__ __forceinline__ T cmk(double re, double im);
template <>
__device__ __forceinline__ double2 cmk<double2>(double re, double im) {
  return make_double2(re, im);
}
template <>
__device__ __forceinline__ float2 cmk<float2>(double re, double im) {
  return make_float2((float)re, (float)im);
}

// ---- bounded grid barrier (all CTAs co-resident: cooperative launch) -------------------
struct GridSync {
  unsigned int* count;
  unsigned int* gen;
  int* status;  // bit 1: barrier timeout
};

__device__ bool grid_barrier(const GridSync& g, unsigned int nblocks) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    volatile unsigned int* vgen = g.gen;
    unsigned int my = *vgen;
    __threadfence();
    unsigned int arrived = atomicAdd(g.count, 1u);
    if (arrived == nblocks - 1) {
      *g.count = 0;
      __threadfence();
      atomicAdd(g.gen, 1u);
    } else {
      long long it = 0;
      while (*vgen == my) {
        if (++it > (1LL << 24)) {  // ~ seconds: give up, report, return
          atomicOr(g.status, 1);
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok;
}

template <typename T>
__device__ __forceinline__ double cabs1(T z) {
  return fabs((double)z.x) + fabs((double)z.y);
}

// ---- panel factorisation ---------------------------------------------------------------
// One CTA per SM keeps its slice of the panel rows in shared memory for the whole panel.
// Per column: local pivot candidate -> publish (value, index, candidate row, and row j if
// owned) into a double-buffered exchange area -> one grid barrier -> every CTA picks the
// same pivot (max |re|+|im|, first index on ties), the owners of rows j and p swap them
// in shared memory, and every CTA scales / rank-1 updates its own rows.
template <typename T>
__global__ void __launch_bounds__(256) k_panel(T* A, int64_t lda, int64_t n, int64_t j0, int nb,
                                               int rows_per, int* ipiv, int* info, double* cand_val,
                                               int* cand_idx, T* cand_row, T* rowj, GridSync gs) {
  extern __shared__ unsigned char smraw[];
  const int ld = nb + 1;  // padded row stride (bank spread)
  T* S = reinterpret_cast<T*>(smraw);              // rows_per x ld
  T* U = S + (size_t)rows_per * ld;                // pivot row (nb)
  __shared__ double sval[256];
  __shared__ int sidx[256];
  __shared__ int s_p;
  __shared__ int s_w[256];
  const unsigned G = gridDim.x;
  const int64_t r0 = j0 + (int64_t)blockIdx.x * rows_per;
  const int nloc = (int)(n - r0 < (int64_t)rows_per ? (n - r0 > 0 ? n - r0 : 0) : (int64_t)rows_per);
  // load own rows of the panel
  for (int e = threadIdx.x; e < nloc * nb; e += blockDim.x) {
    int i = e % nloc, k = e / nloc;
    S[i * ld + k] = A[(r0 + i) + (j0 + k) * lda];
  }
  __syncthreads();
  for (int jj = 0; jj < nb; ++jj) {
    const int64_t j = j0 + jj;
    const int buf = jj & 1;
    // 1. local candidate over own rows with global index >= j
    double bv = -1.0;
    int bi = 0x7fffffff;
    for (int i = threadIdx.x; i < nloc; i += blockDim.x) {
      if (r0 + i < j) continue;
      T a = S[i * ld + jj];
      double v = fabs((double)a.x) + fabs((double)a.y);
      if (v > bv) {
        bv = v;
        bi = i;
      }
    }
    sval[threadIdx.x] = bv;
    sidx[threadIdx.x] = bi;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
      if (threadIdx.x < o) {
        double v2 = sval[threadIdx.x + o];
        int i2 = sidx[threadIdx.x + o];
        if (v2 > sval[threadIdx.x] || (v2 == sval[threadIdx.x] && i2 < sidx[threadIdx.x])) {
          sval[threadIdx.x] = v2;
          sidx[threadIdx.x] = i2;
        }
      }
      __syncthreads();
    }
    const int li = sidx[0];
    if (threadIdx.x == 0) {
      cand_val[buf * G + blockIdx.x] = sval[0];
      cand_idx[buf * G + blockIdx.x] = sval[0] >= 0.0 ? (int)(r0 + li) : 0x7fffffff;
    }
    if (sval[0] >= 0.0)
      for (int k = threadIdx.x; k < nb; k += blockDim.x)
        cand_row[((size_t)buf * G + blockIdx.x) * nb + k] = S[li * ld + k];
    const bool own_j = (j >= r0 && j < r0 + nloc);
    if (own_j)
      for (int k = threadIdx.x; k < nb; k += blockDim.x) rowj[(size_t)buf * nb + k] = S[(j - r0) * ld + k];
    if (!grid_barrier(gs, G)) return;
    // 2. global pivot: the G candidates are read in parallel and reduced in shared memory
    {
      double v = -1.0;
      int p = 0x7fffffff, w = 0;
      for (unsigned b = threadIdx.x; b < G; b += blockDim.x) {
        double cv = __ldcg(cand_val + buf * G + b);
        int ci = __ldcg(cand_idx + buf * G + b);
        if (cv > v || (cv == v && ci < p)) {
          v = cv;
          p = ci;
          w = (int)b;
        }
      }
      __syncthreads();  // everyone has read li / sidx of step 1
      sval[threadIdx.x] = v;
      sidx[threadIdx.x] = p;
      s_w[threadIdx.x] = w;
      __syncthreads();
      for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
          double v2 = sval[threadIdx.x + o];
          int i2 = sidx[threadIdx.x + o];
          if (v2 > sval[threadIdx.x] || (v2 == sval[threadIdx.x] && i2 < sidx[threadIdx.x])) {
            sval[threadIdx.x] = v2;
            sidx[threadIdx.x] = i2;
            s_w[threadIdx.x] = s_w[threadIdx.x + o];
          }
        }
        __syncthreads();
      }
    }
    if (threadIdx.x == 0) {
      double v = sval[0];
      int p = sidx[0], w = s_w[0];
      if (v <= 0.0) {  // exactly singular column: record, no interchange
        p = (int)j;
        w = -1;
        if (blockIdx.x == 0 && *info == 0) *info = (int)j + 1;
      }
      if (blockIdx.x == 0) ipiv[j] = p;
      s_p = p;
      sidx[0] = w;
    }
    __syncthreads();
    const int64_t p = s_p;
    const int wblk = sidx[0];
    if (wblk < 0) {
      for (int k = threadIdx.x; k < nb; k += blockDim.x) U[k] = own_j ? S[(j - r0) * ld + k] : __ldcg(rowj + (size_t)buf * nb + k);
    } else {
      for (int k = threadIdx.x; k < nb; k += blockDim.x)
        U[k] = __ldcg(cand_row + ((size_t)buf * G + wblk) * nb + k);
    }
    __syncthreads();
    // the owners exchange rows j and p (row p receives row j's content)
    if (p != j) {
      if (p >= r0 && p < r0 + nloc)
        for (int k = threadIdx.x; k < nb; k += blockDim.x) S[(p - r0) * ld + k] = __ldcg(rowj + (size_t)buf * nb + k);
      __syncthreads();
      if (own_j)
        for (int k = threadIdx.x; k < nb; k += blockDim.x) S[(j - r0) * ld + k] = U[k];
    }
    __syncthreads();
    // 3. scale and rank-1 update of own rows below j
    T piv = U[jj];
    double den = (double)piv.x * piv.x + (double)piv.y * piv.y;
    if (den != 0.0) {
      typedef decltype(piv.x) RT;
      const RT ir = (RT)(piv.x / den), ii = (RT)(-piv.y / den);
      const int ncol = nb - jj - 1;
      const int64_t ibeg = (j + 1 - r0) > 0 ? (j + 1 - r0) : 0;
      for (int64_t i = ibeg + threadIdx.x; i < nloc; i += blockDim.x) {  // multipliers
        T a = S[i * ld + jj];
        T l;
        l.x = a.x * ir - a.y * ii;
        l.y = a.x * ii + a.y * ir;
        S[i * ld + jj] = l;
      }
      __syncthreads();
      for (int64_t e = threadIdx.x; e < (nloc - ibeg) * (int64_t)ncol; e += blockDim.x) {
        int i = (int)(ibeg + e / ncol);
        int k = jj + 1 + (int)(e % ncol);
        T l = S[i * ld + jj];
        T u = U[k];
        T c = S[i * ld + k];
        c.x -= l.x * u.x - l.y * u.y;
        c.y -= l.x * u.y + l.y * u.x;
        S[i * ld + k] = c;
      }
    }
    __syncthreads();
  }
  // write back
  for (int e = threadIdx.x; e < nloc * nb; e += blockDim.x) {
    int i = e % nloc, k = e / nloc;
    A[(r0 + i) + (j0 + k) * lda] = S[i * ld + k];
  }
}

// ---- row interchanges ipiv[p0, p1) applied (in order) to columns [c0, c1) ----------------
template <typename T>
__global__ void k_laswp(T* A, int64_t lda, int64_t c0, int64_t c1, int64_t p0, int64_t p1,
                        const int* ipiv) {
  int64_t col = c0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (col >= c1) return;
  for (int64_t r = p0; r < p1; ++r) {
    int64_t p = ipiv[r];
    if (p != r) {
      T a = A[r + col * lda];
      A[r + col * lda] = A[p + col * lda];
      A[p + col * lda] = a;
    }
  }
}

// ---- LU of a diagonal block without pivoting (mixed path) --------------------------------
// A[j0:j0+kb, j0:j0+kb] = L11 U11 in place, kb <= 64, one CTA of 256 threads in shared
// memory, blocked by 16 columns (three barriers per 16 pivots):
//   1. warp 0 factors the 64 x 16 column slab in registers (lane l holds rows l and l + 32;
//      the pivot row is broadcast with shuffles, so the 16 pivot steps need no block barrier);
//   2. U12 of the slab's rows, one column per thread (unit lower 16 x 16 substitution);
//   3. rank-16 update of the trailing block by all threads.
// A zero pivot sets *info (1-based column) and the kernel stops.
constexpr int TRI = 64;

template <typename T>
__device__ __forceinline__ void cfms(T& acc, T a, T b) {  // acc -= a b, four fused multiply-adds
  acc.x = fma(-a.x, b.x, acc.x);
  acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(-a.x, b.y, acc.y);
  acc.y = fma(-a.y, b.x, acc.y);
}
template <typename T>
__device__ __forceinline__ void cfma(T& acc, T a, T b) {  // acc += a b
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
}
template <typename T>
__device__ __forceinline__ T cmulx(T a, T b) {
  T r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
// r = 1 / p; false for p = 0.  FP32: the hardware reciprocal (rcp.approx, within 1 ulp) --
// this is on the serial pivot chain of the unpivoted mixed-precision LU, whose result is
// refined in FP64 anyway; FP64: IEEE division
__device__ __forceinline__ float rcp_f(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ bool crecip(float2 p, float2& r) {
  const float den = p.x * p.x + p.y * p.y;
  if (den == 0.f) return false;
  const float id = rcp_f(den);
  r.x = p.x * id;
  r.y = -p.y * id;
  return true;
}
__device__ __forceinline__ bool crecip(double2 p, double2& r) {
  const double den = p.x * p.x + p.y * p.y;
  if (den == 0.0) return false;
  const double id = 1.0 / den;
  r.x = p.x * id;
  r.y = -p.y * id;
  return true;
}

template <typename T>
__device__ __forceinline__ T shfl_c(T v, int src) {
  T r;
  r.x = __shfl_sync(0xffffffffu, v.x, src);
  r.y = __shfl_sync(0xffffffffu, v.y, src);
  return r;
}

template <typename T>
__global__ void __launch_bounds__(256) k_getrf64(T* A, int64_t lda, int64_t j0, int kb, int* info) {
  constexpr int LD = TRI + 1, PB = 16;
  extern __shared__ unsigned char smraw[];
  T* D = reinterpret_cast<T*>(smraw);  // row-major, ld LD, zero outside kb x kb
  __shared__ int s_zero;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // the block, 16 loads per thread issued before their stores so that they overlap
  {
    T v[TRI * TRI / 256];
#pragma unroll
    for (int j = 0; j < TRI * TRI / 256; ++j) {
      const int e = tid + 256 * j, r = e % TRI, k = e / TRI;
      v[j] = (r < kb && k < kb) ? A[(j0 + r) + (j0 + k) * lda] : T{0, 0};
    }
#pragma unroll
    for (int j = 0; j < TRI * TRI / 256; ++j) {
      const int e = tid + 256 * j;
      D[(e % TRI) * LD + e / TRI] = v[j];
    }
  }
  if (tid == 0) s_zero = 0;
  __syncthreads();
  for (int k0 = 0; k0 < kb; k0 += PB) {
    const int nbk = min(PB, kb - k0);
    // 1. the column slab k0 .. k0+15 by warp 0
    if (warp == 0) {
      T a[2][PB];
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int c = 0; c < PB; ++c) a[h][c] = D[(lane + 32 * h) * LD + k0 + c];
      int zero_at = 0;
#pragma unroll
      for (int k = 0; k < PB; ++k) {
        if (k < nbk && zero_at == 0) {  // uniform over the warp
          const int pr = k0 + k, ow = pr & 31, oh = pr >> 5;
          T u[PB];
#pragma unroll
          for (int c = k; c < PB; ++c) u[c] = shfl_c(oh ? a[1][c] : a[0][c], ow);
          T ip;
          if (!crecip(u[k], ip)) {
            zero_at = pr + 1;
          } else {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              const int i = lane + 32 * h;
              if (i > pr && i < kb) {
                const T l = cmulx(a[h][k], ip);
                a[h][k] = l;
#pragma unroll
                for (int c = k + 1; c < PB; ++c) cfms(a[h][c], l, u[c]);
              }
            }
          }
        }
      }
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int c = 0; c < PB; ++c) D[(lane + 32 * h) * LD + k0 + c] = a[h][c];
      if (lane == 0 && zero_at) s_zero = zero_at;
    }
    __syncthreads();
    if (s_zero) {  // uniform
      if (tid == 0) atomicCAS(info, 0, (int)(j0 + s_zero));
      return;
    }
    const int c1 = k0 + PB;  // first column right of the slab (the slab is complete here)
    if (c1 >= kb) break;
    // 2. U12 = L11^{-1} A12 for the slab's 16 rows, one column per thread
    if (tid < kb - c1) {
      const int c = c1 + tid;
      T x[PB];
#pragma unroll
      for (int i = 0; i < PB; ++i) x[i] = D[(k0 + i) * LD + c];
#pragma unroll
      for (int i = 1; i < PB; ++i)
#pragma unroll
        for (int j = 0; j < i; ++j) cfms(x[i], D[(k0 + i) * LD + k0 + j], x[j]);
#pragma unroll
      for (int i = 1; i < PB; ++i) D[(k0 + i) * LD + c] = x[i];
    }
    __syncthreads();
    // 3. rank-16 update of the trailing block
    const int w = kb - c1;
    for (int e = tid; e < w * w; e += 256) {
      const int r = c1 + e / w, c = c1 + e % w;
      T acc = D[r * LD + c];
#pragma unroll
      for (int j = 0; j < PB; ++j) cfms(acc, D[r * LD + k0 + j], D[(k0 + j) * LD + c]);
      D[r * LD + c] = acc;
    }
    __syncthreads();
  }
  for (int e = tid; e < kb * kb; e += 256) {
    const int r = e % kb, k = e / kb;
    A[(j0 + r) + (j0 + k) * lda] = D[r * LD + k];
  }
}

// ---- diagonal block LU together with the inverses of its triangles ---------------------
// For the unpivoted c64 path: the 64 x 64 block at (j0, j0) (kb x kb, the rest padded with
// the identity) is factored by forward elimination on [A | I] -- eliminating below the pivot
// turns the identity part of the rows into L^{-1} (it lives in the strictly lower positions
// the elimination has just emptied), while the upper part becomes U -- and in the same pass
// X = (U^T)^{-1} = (U^{-1})^T is built by forward elimination on U^T, whose multipliers
// U[k][r] are the pivot row itself.  Step k (rows r > k), with d = 1 / U[k][k]:
//   S1[r][c] -= (A[r][k] d) P1[c]   (P1 = row k of S1 with 0 at column k)
//   S1[r][k]  = -A[r][k] d          (L^{-1}[r][k] after this step; L[r][k] = A[r][k] d)
//   S2[r][c] -= (U[k][r] d) P2[c]   (P2 = row k of S2, before its own scaling)
//   S2[k][c] *= d
// Each thread holds a 4 x 4 tile of S1 and of S2 in registers (rows 4 rb.., columns 4 cb..;
// a warp = 2 row blocks x 16 column blocks).  After each step the owners of row k+1, of
// column k+1 and of the pivot publish P1, P2, the column and 1 / pivot in shared memory
// (double-buffered by step parity): one block barrier per step.  The step loop is unrolled
// by 4, so the tile slot of row / column k is known at compile time and the code is short
// (this kernel runs alone on one SM between wide launches: it is latency-bound and starts
// with cold instruction caches).  Output: the factors in A, Linv and Uinv (column-major
// 64 x 64, identity beyond kb) in inv.  A zero pivot sets *info (1-based column) and the
// kernel stops.
template <typename T>
__device__ __forceinline__ int pidx(int c) {  // conflict-free index of the published rows
  return c + (c >> 2);
}

// SYM: only the lower triangle of the block is current (symmetric updates); the upper one
// is taken from it by symmetry, the elimination on U^T is skipped and, U = D L^T,
// U^{-1} = (L^{-1})^T D^{-1} is formed from L^{-1} and the pivots at the end.
// TR x TC: the tile a thread owns (rows x columns): 4 x 4 (256 threads), 2 x 4 (512) or 2 x 2
// (1024 threads: a quarter of the serial instructions per warp and step of 4 x 4, which is what
// bounds this latency-bound chain).  The arithmetic per element is the same for every tile.
template <typename T, bool SYM, int TR = 4, int TC = TR>
__global__ void __launch_bounds__(TRI * TRI / (TR * TC)) k_lu_inv64(T* A, int64_t lda, int64_t j0, int kb, int* info,
                                                                   T* inv) {
  constexpr bool sym = SYM;
  constexpr int NT = TRI * TRI / (TR * TC);  // threads
  constexpr int NCB = TRI / TC;              // column blocks: 32 (a warp) or 16 (half a warp)
  static_assert(TC % TR == 0 && (NCB == 32 || NCB == 16), "tile: TR divides TC, TC = 2 or 4");
  constexpr int LD = TRI + 1, PL = TRI + TRI / 4;
  extern __shared__ unsigned char smraw[];
  T* Ls = reinterpret_cast<T*>(smraw);  // 64 x LD: staging, then the L factor, then Linv
  __shared__ T p1[2][PL], p2[2][PL], lc[2][TRI];
  __shared__ T dv[2];
  __shared__ int s_zero[2];  // 1-based column of a zero pivot, by step parity
  // the panel products launched after this kernel may start their loads now (they wait for
  // its results before reading them)
  asm volatile("griddepcontrol.launch_dependents;");
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int cb = NCB == 16 ? (lane & 15) : lane, rb = NCB == 16 ? 2 * warp + (lane >> 4) : warp;
  const int r0 = TR * rb, c0 = TC * cb;
  const T zero = cmk<T>(0.0, 0.0), one = cmk<T>(1.0, 0.0);
  // coalesced load through shared memory (identity padding beyond kb)
  for (int e = tid; e < TRI * TRI; e += NT) {
    const int r = e & (TRI - 1), c = e >> 6;
    const int rr = (sym && c > r) ? c : r, cc = (sym && c > r) ? r : c;
    Ls[r * LD + c] = (r < kb && c < kb) ? A[(j0 + rr) + (j0 + cc) * lda] : (r == c ? one : zero);
  }
  if (tid < 2) s_zero[tid] = 0;
  __syncthreads();
  T s1[TR][TC], s2[TR][TC];
#pragma unroll
  for (int i = 0; i < TR; ++i)
#pragma unroll
    for (int j = 0; j < TC; ++j) {
      s1[i][j] = Ls[(r0 + i) * LD + c0 + j];
      s2[i][j] = (r0 + i == c0 + j) ? one : zero;
    }
  // publish row 0, column 0 and the first pivot's reciprocal
  if (rb == 0)
#pragma unroll
    for (int j = 0; j < TC; ++j) {
      p1[0][pidx<T>(c0 + j)] = (c0 + j == 0) ? zero : s1[0][j];
      if (!SYM) p2[0][pidx<T>(c0 + j)] = s2[0][j];
    }
  if (cb == 0)
#pragma unroll
    for (int i = 0; i < TR; ++i) lc[0][r0 + i] = s1[i][0];
  if (rb == 0 && cb == 0) {
    T d;
    if (!crecip(s1[0][0], d)) s_zero[0] = 1;
    dv[0] = d;
  }
  __syncthreads();  // the staging buffer is free from here on (L factor)
  // steps unrolled by TC: column k is slot kk of column block kq, row k slot kk % TR of row
  // block k / TR (TR divides TC), so every register index below is known at compile time
  for (int kq = 0; kq < TRI / TC; ++kq) {
#pragma unroll
    for (int kk = 0; kk < TC; ++kk) {
      const int k = TC * kq + kk, b = kk & 1;
      if (s_zero[b]) {  // uniform
        if (tid == 0) atomicCAS(info, 0, (int)(j0 + s_zero[b]));
        return;
      }
      const T d = dv[b];
      if (r0 + TR - 1 > k) {  // some row of the tile is below the pivot
        T l1[TR], l2[TR], q1[TC], q2[TC];
#pragma unroll
        for (int i = 0; i < TR; ++i) {
          l1[i] = cmulx(lc[b][r0 + i], d);
          l2[i] = cmulx(p1[b][pidx<T>(r0 + i)], d);
        }
#pragma unroll
        for (int j = 0; j < TC; ++j) {
          q1[j] = p1[b][pidx<T>(c0 + j)];
          q2[j] = p2[b][pidx<T>(c0 + j)];
        }
#pragma unroll
        for (int i = 0; i < TR; ++i)
          if (r0 + i > k) {
#pragma unroll
            for (int j = 0; j < TC; ++j) {
              cfms(s1[i][j], l1[i], q1[j]);
              if (!SYM) cfms(s2[i][j], l2[i], q2[j]);
            }
            if (cb == kq) {  // column k: L^{-1}[r][k] = -l, and the L factor
              s1[i][kk].x = -l1[i].x;
              s1[i][kk].y = -l1[i].y;
              Ls[(r0 + i) * LD + k] = l1[i];
            }
          }
      }
      if (!SYM && rb == k / TR)  // row k of X is final
#pragma unroll
        for (int j = 0; j < TC; ++j) s2[kk % TR][j] = cmulx(s2[kk % TR][j], d);
      // publish step k + 1
      if (k + 1 < TRI) {
        const int kn = k + 1, bn = b ^ 1;
        const int qr = kn / TR, ir = (kk + 1) % TR, qc = kn / TC, ic = (kk + 1) % TC;
        if (rb == qr)
#pragma unroll
          for (int j = 0; j < TC; ++j) {
            p1[bn][pidx<T>(c0 + j)] = (c0 + j == kn) ? zero : s1[ir][j];
            if (!SYM) p2[bn][pidx<T>(c0 + j)] = s2[ir][j];
          }
        if (cb == qc)
#pragma unroll
          for (int i = 0; i < TR; ++i) lc[bn][r0 + i] = s1[i][ic];
        if (rb == qr && cb == qc) {
          T dn;
          if (!crecip(s1[ir][ic], dn)) s_zero[bn] = kn + 1;
          dv[bn] = dn;
        }
      }
      __syncthreads();
    }
  }
  // U (upper part of S1) joins the L factor in Ls; the factored block goes back to A
#pragma unroll
  for (int i = 0; i < TR; ++i)
#pragma unroll
    for (int j = 0; j < TC; ++j)
      if (c0 + j >= r0 + i) Ls[(r0 + i) * LD + c0 + j] = s1[i][j];
  __syncthreads();
  for (int e = tid; e < kb * kb; e += NT) {
    const int r = e % kb, c = e / kb;
    A[(j0 + r) + (j0 + c) * lda] = Ls[r * LD + c];
  }
  __syncthreads();
  // Linv (column-major, inv[c * 64 + r] = Linv[r][c]) through Ls; Uinv = X^T, so row r of X
  // is column r of Uinv (inv[4096 + r * 64 + c] = X[r][c]), written by the tile owners;
  // symmetric: X[r][c] = Linv[r][c] / d_r
  if (SYM) {
    __shared__ T s_dinv[TRI];
#pragma unroll
    for (int i = 0; i < TR; ++i)
#pragma unroll
      for (int j = 0; j < TC; ++j)
        if (c0 + j == r0 + i) {  // the tile holding the pivot of row r0 + i
          T di;
          crecip(s1[i][j], di);  // nonzero: the elimination checked every pivot
          s_dinv[r0 + i] = di;
        }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < TR; ++i) {
      const T di = s_dinv[r0 + i];
#pragma unroll
      for (int j = 0; j < TC; ++j) {
        const int r = r0 + i, c = c0 + j;
        s2[i][j] = c < r ? cmulx(s1[i][j], di) : (c == r ? di : zero);
      }
    }
  }
#pragma unroll
  for (int i = 0; i < TR; ++i)
#pragma unroll
    for (int j = 0; j < TC; ++j) {
      const int r = r0 + i, c = c0 + j;
      Ls[r * LD + c] = c < r ? s1[i][j] : (c == r ? one : zero);
      inv[TRI * TRI + r * TRI + c] = s2[i][j];
    }
  __syncthreads();
  for (int e = tid; e < TRI * TRI; e += NT) {
    const int r = e & (TRI - 1), c = e >> 6;
    inv[e] = Ls[r * LD + c];
  }
}

// ---- blocked triangular solves on 64-wide triangles ---------------------------------------
// Both TRSMs of the LU are batches of independent triangular systems of order kb <= 64 that
// share one triangle of the factored diagonal block at (j0, j0):
//   left  (U12 = L11^{-1} A12): one system per column of A12, unit lower L11;
//   right (unpivoted path, L21 = A21 U11^{-1}): one system per row of A21, upper U11.
// A CTA stages NS = 64 systems (coalesced global loads) as X[k][s] in shared memory and the
// triangle as M[k][c] = coefficient of x_k in equation c (k < c).  Four neighbouring lanes
// share a system and substitute in blocks of 16 unknowns, lane j of the four owning unknowns
// 4j .. 4j+3 of each block:
//   x_c = (a_c - sum_{k<c} M[k][c] x_k) * d_c     (d_c = 1 or 1/U_cc);
// the terms of earlier blocks are split over the four lanes, and inside a block each solved
// unknown is passed to the other three lanes by a shuffle.
template <typename T>
struct TrsmTile {
  static constexpr int NS = 64;                          // systems per CTA
  static constexpr int NT = 4 * NS;                      // threads per CTA
  static constexpr int MLD = sizeof(T) == 8 ? 66 : 65;   // row stride of M
};

template <typename T>
size_t trsm_tile_smem() {
  return ((size_t)TRI * TrsmTile<T>::MLD + TRI + (size_t)TRI * (TrsmTile<T>::NS + 1)) * sizeof(T);
}

template <typename T, typename RT, bool RIGHT>
__global__ void __launch_bounds__(TrsmTile<T>::NT) k_trsm_tile(T* A, int64_t lda, int64_t j0, int kb,
                                                               int64_t s0, int64_t s1) {
  constexpr int NS = TrsmTile<T>::NS, NT = TrsmTile<T>::NT, MLD = TrsmTile<T>::MLD, LDX = NS + 1;
  extern __shared__ __align__(16) unsigned char smraw[];
  T* M = reinterpret_cast<T*>(smraw);  // TRI x MLD
  T* dinv = M + TRI * MLD;             // TRI
  T* X = dinv + TRI;                   // TRI x LDX
  const int tid = threadIdx.x;
  const int64_t sb = s0 + (int64_t)blockIdx.x * NS;  // first system of this CTA
  const T zero = {0, 0};

  // the triangle (zero outside kb x kb and on/below the diagonal of M) and the systems
  // X[k][s]; each thread issues its 16 + 16 loads before the stores
  constexpr int LB = TRI * TRI / NT;
  static_assert(LB * NT == TRI * TRI && LB * NT == TRI * NS, "staging");
  {
    T v[LB];
#pragma unroll
    for (int j = 0; j < LB; ++j) {
      const int e = tid + NT * j;
      const int r = e % TRI, k = e / TRI;  // global element (j0 + r, j0 + k), coalesced along r
      v[j] = (r < kb && k < kb) ? A[(j0 + r) + (j0 + k) * lda] : zero;
    }
#pragma unroll
    for (int j = 0; j < LB; ++j) {
      const int e = tid + NT * j;
      const int r = e % TRI, k = e / TRI;
      if (RIGHT) {
        M[r * MLD + k] = r < k ? v[j] : zero;  // U[r][k]: coefficient of x_r in equation k
        if (r == k) {
          T d = zero;
          if (r < kb) {
            const RT den = v[j].x * v[j].x + v[j].y * v[j].y;
            d.x = v[j].x / den;
            d.y = -v[j].y / den;
          }
          dinv[r] = d;
        }
      } else {
        M[k * MLD + r] = r > k ? v[j] : zero;  // L[r][k]: coefficient of x_k in equation r
      }
    }
  }
  {
    T v[LB];
#pragma unroll
    for (int j = 0; j < LB; ++j) {
      const int e = tid + NT * j;
      if (RIGHT) {
        const int s = e % NS, k = e / NS;  // row sb + s, column j0 + k: coalesced along s
        v[j] = (k < kb && sb + s < s1) ? A[(sb + s) + (j0 + k) * lda] : zero;
      } else {
        const int k = e % TRI, s = e / TRI;  // row j0 + k, column sb + s: coalesced along k
        v[j] = (k < kb && sb + s < s1) ? A[(j0 + k) + (sb + s) * lda] : zero;
      }
    }
#pragma unroll
    for (int j = 0; j < LB; ++j) {
      const int e = tid + NT * j;
      if (RIGHT)
        X[(e / NS) * LDX + e % NS] = v[j];
      else
        X[(e % TRI) * LDX + e / TRI] = v[j];
    }
  }
  __syncthreads();

  // substitution: lane quad (4 s .. 4 s + 3) of the warp owns system s, lane j owns
  // unknowns 4 j .. 4 j + 3 of each block of 16
  const int s = tid >> 2, j = tid & 3, qbase = (tid & 31) & ~3;
  T* x = X + s;
  const int nblk = (kb + 15) / 16;
  for (int B = 0; B < nblk; ++B) {
    const int c0 = 16 * B, cj = c0 + 4 * j;
    T acc[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) acc[i] = x[(cj + i) * LDX];
    // c0 is a multiple of 16: four earlier unknowns per pass, their loads issued together
    for (int k = 0; k < c0; k += 4) {
      T xk[4], mk[4][4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        xk[u] = x[(k + u) * LDX];
#pragma unroll
        for (int i = 0; i < 4; ++i) mk[u][i] = M[(k + u) * MLD + cj + i];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int i = 0; i < 4; ++i) cfms(acc[i], mk[u][i], xk[u]);
    }
#pragma unroll
    for (int cc = 0; cc < 16; ++cc) {
      const int jo = cc >> 2, io = cc & 3;
      if (RIGHT && j == jo) {
        const T d = dinv[c0 + cc];
        acc[io] = cmulx(acc[io], d);
      }
      const T xc = shfl_c(acc[io], qbase + jo);  // the solved unknown c0 + cc
      if (j == jo) x[(c0 + cc) * LDX] = xc;
#pragma unroll
      for (int i = 0; i < 4; ++i)
        if (4 * j + i > cc) cfms(acc[i], M[(c0 + cc) * MLD + cj + i], xc);
    }
  }
  __syncthreads();

  // write the solved systems back
  for (int m0 = 0; m0 < TRI * NS / NT; ++m0) {
    const int e = tid + NT * m0;
    if (RIGHT) {
      const int s2 = e % NS, k = e / NS;
      if (k < kb && sb + s2 < s1) A[(sb + s2) + (j0 + k) * lda] = X[k * LDX + s2];
    } else {
      const int k = e % TRI, s2 = e / TRI;
      if (k < kb && sb + s2 < s1) A[(j0 + k) + (sb + s2) * lda] = X[k * LDX + s2];
    }
  }
}

// ---- unpivoted c64 panel: both triangular solves as products with the inverses ----------
// After k_lu_inv64 (kb = 64, inverses in inv: Linv then Uinv, column-major 64 x 64), with
// s0 = j0 + 64:
//   CTA b <  nR:  L21 rows s0 + 64 b .. +63:          X = A21 Uinv  (a system per row)
//   CTA b >= nR:  U12 columns s0 + 64 (b - nR) .. +63: X = Linv A12  (a system per column)
// Both are C[x][y] = sum_k W[k][s] N[k][v] over 64 x 64 x 64: s runs over the 64 systems
// (W: A21 / A12), v over the inverse's free index (N: Uinv / Linv), and N[k][v] = 0 for
// k > v (the triangle).  A complex multiply-add is two packed FP32 FMAs,
//   acc += (a.x, a.x) (b.x, b.y) + (-a.y, a.y) (b.y, b.x),
// so W is staged as float4 (a.x, a.x, -a.y, a.y) and N as float4 (b.x, b.y, b.y, b.x): one
// 16-byte load per operand and no register shuffling.  K is staged in two halves of 32.
// A thread owns 4 systems (lanes 0..15 of a half-warp at stride 16) times 4 free indices,
// dealt out so that every warp does the same work: warp w takes 4w .. 4w+3 and
// 60-4w .. 63-4w (half-warp h the pairs at +2h), all four up to k = 4w+4, the upper two up
// to 64-4w -- 544 complex multiply-adds per thread in every warp.  The result is staged
// system-major in shared memory, stored coalesced and, when the tensor-core update follows
// (Ap / Bp not null), written once more as its FP16 operands with 16-byte stores: L21 rows
// expanded and row-scaled as A', U12 columns scaled as B' (layout and scale rule of the
// update's own operand preparation).
constexpr int PA_KH = 32;   // k per staged half
constexpr int PA_LD4 = 65;  // staged operand rows: 64 float4 + 1
constexpr int PA_CLD = 65;  // staged result columns
size_t panel_apply_smem() { return (size_t)2 * PA_KH * PA_LD4 * sizeof(float4) + 4 * 64 * sizeof(float); }

__device__ __forceinline__ void cmac2(float2& acc, float4 a, float4 b) {
  acc = __ffma2_rn(make_float2(a.x, a.y), make_float2(b.x, b.y), acc);
  acc = __ffma2_rn(make_float2(a.z, a.w), make_float2(b.z, b.w), acc);
}

// Symmetric factorisation (nB >= 0; launched with nR CTAs, right side only): U12 = D L21^T
// is not stored; its FP16 B' columns for the first nB systems (the rest of the mid block)
// are written from L21 and the pivots D = diag(U11) instead.
// rb0: index of the first CTA's block (the grid covers blocks rb0 .. of the 2 nR, or nR)
template <int NS>
__global__ void __launch_bounds__(256, NS == 64 ? 2 : 3) k_panel_apply(float2* A, int64_t lda, int64_t j0, int64_t n,
                                                        const float2* inv, int nR, __half2* Ap,
                                                        float* inv_sa, __half2* Bp, float* inv_sb, int nB,
                                                        int rb0) {
  extern __shared__ __align__(16) unsigned char smraw[];
  float4* Ws = reinterpret_cast<float4*>(smraw);  // W[k][s], k of the current half
  float4* Ns = Ws + PA_KH * PA_LD4;               // N[k][v]
  float* red = reinterpret_cast<float*>(Ns + PA_KH * PA_LD4);  // 4 x 64 partial maxima
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int bi = (int)blockIdx.x + rb0;
  const bool right = bi < nR;
  const int64_t s0 = j0 + TRI;
  const int64_t b0 = s0 + (int64_t)(right ? bi : bi - nR) * NS;  // first system
  constexpr int NU = NS / 16;         // systems per thread
  constexpr int QN = 256 / NS;        // threads per system in the maxima passes
  constexpr int QV = TRI / QN;        // free indices per such thread
  const float2 zero = make_float2(0.f, 0.f);
  const int sl = lane & 15, h = lane >> 4;
  const int vlo = 4 * warp + 2 * h, vhi = 60 - 4 * warp + 2 * h;  // free indices vlo, vlo+1, vhi, vhi+1
  const int k1 = 4 * warp + 4, k2 = 64 - 4 * warp;
  float2 acc[NU][4];  // [system u][free index: vlo, vlo+1, vhi, vhi+1]
#pragma unroll
  for (int u = 0; u < NU; ++u)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[u][j] = zero;

  for (int kh = 0; kh < 2; ++kh) {
    const int kb0 = kh * PA_KH;
    if (kh) __syncthreads();  // the first half is consumed
    {
      // 8 + 8 elements per thread, e = tid + 256 t; coalesced along the contiguous index:
      //   right W: s = e & 63, k = e >> 6 (A21 column k)   N: k = e & 31, v = e >> 5 (Uinv column v)
      //   left  W: k = e & 31, s = e >> 5 (A12 column s)   N: v = e & 63, k = e >> 6 (Linv column k)
      constexpr int TW = NS * PA_KH / 256;  // W elements per thread (N: 8)
      float2 w[TW], v[8];
#pragma unroll
      for (int t = 0; t < TW; ++t) {
        const int e = tid + 256 * t;
        if (right) {
          const int s = e % NS, k = e / NS;
          w[t] = b0 + s < n ? A[(b0 + s) + (j0 + kb0 + k) * lda] : zero;
        } else {
          const int k = e & 31, s = e >> 5;
          w[t] = b0 + s < n ? A[(j0 + kb0 + k) + (b0 + s) * lda] : zero;
        }
      }
      // launched as a programmatic dependent of the diagonal block's elimination: the rows of
      // A21 / A12 above are final already, the inverses (and the pivots below) only after this
      // wait (a no-op for an ordinary launch); `inv` is not declared __restrict__ and is read
      // through L2, so that no load of it is scheduled or served from before the wait
      if (kh == 0) asm volatile("griddepcontrol.wait;" ::: "memory");
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const int e = tid + 256 * t;
        v[t] = __ldcg(right ? inv + 4096 + (e >> 5) * 64 + kb0 + (e & 31) : inv + (kb0 + (e >> 6)) * 64 + (e & 63));
      }
#pragma unroll
      for (int t = 0; t < TW; ++t) {
        const int e = tid + 256 * t;
        const float4 wv = make_float4(w[t].x, w[t].x, -w[t].y, w[t].y);
        if (right)
          Ws[(e / NS) * PA_LD4 + (e % NS)] = wv;
        else
          Ws[(e & 31) * PA_LD4 + (e >> 5)] = wv;
      }
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const int e = tid + 256 * t;
        const float4 nv = make_float4(v[t].x, v[t].y, v[t].y, v[t].x);
        if (right)
          Ns[(e & 31) * PA_LD4 + (e >> 5)] = nv;
        else
          Ns[(e >> 6) * PA_LD4 + (e & 63)] = nv;
      }
    }
    __syncthreads();
    // all four free indices for k < k1 (inside the first half), the upper two for k < k2
    const int e1 = kh == 0 ? k1 : kb0, e2 = min(k2, kb0 + PA_KH);
#pragma unroll 2
    for (int k = kb0; k < e1; ++k) {
      const float4* wr = Ws + (k - kb0) * PA_LD4 + sl;
      const float4* nr = Ns + (k - kb0) * PA_LD4;
      const float4 n0 = nr[vlo], n1 = nr[vlo + 1], n2 = nr[vhi], n3 = nr[vhi + 1];
#pragma unroll
      for (int u = 0; u < NU; ++u) {
        const float4 a = wr[16 * u];
        cmac2(acc[u][0], a, n0);
        cmac2(acc[u][1], a, n1);
        cmac2(acc[u][2], a, n2);
        cmac2(acc[u][3], a, n3);
      }
    }
#pragma unroll 2
    for (int k = e1; k < e2; ++k) {
      const float4* wr = Ws + (k - kb0) * PA_LD4 + sl;
      const float4* nr = Ns + (k - kb0) * PA_LD4;
      const float4 n2 = nr[vhi], n3 = nr[vhi + 1];
#pragma unroll
      for (int u = 0; u < NU; ++u) {
        const float4 a = wr[16 * u];
        cmac2(acc[u][2], a, n2);
        cmac2(acc[u][3], a, n3);
      }
    }
  }
  __syncthreads();  // every warp is done with Ws / Ns
  // stage C system-major, Cs[s][v] (s: system, v: free index)
  float2* Cs = reinterpret_cast<float2*>(smraw);
  __shared__ float s_scale[64];
  const int vv[4] = {vlo, vlo + 1, vhi, vhi + 1};
#pragma unroll
  for (int u = 0; u < NU; ++u)
#pragma unroll
    for (int j = 0; j < 4; ++j) Cs[(sl + 16 * u) * PA_CLD + vv[j]] = acc[u][j];
  __syncthreads();
  // the solved systems, coalesced: right -- A[b0 + s, j0 + v] (along s); left -- A[j0 + v,
  // b0 + s] (along v)
#pragma unroll 4
  for (int t = 0; t < NS / 4; ++t) {
    const int e = tid + 256 * t;
    if (right) {
      const int sy = e % NS, v = e / NS;
      if (b0 + sy < n) A[(b0 + sy) + (j0 + v) * lda] = Cs[sy * PA_CLD + v];
    } else {
      const int v = e & 63, sy = e >> 6;
      if (b0 + sy < n) A[(j0 + v) + (b0 + sy) * lda] = Cs[sy * PA_CLD + v];
    }
  }
  // FP16 operands of the update: right -- the A' row pair of each system (2 x 64 half2);
  // left -- the B' column of each system (64 half2).  Scale: 2^sh from the system's largest
  // |re|, |im| (partial maxima over quarters of v, then one per system).
  __half2* const dst = right ? Ap : Bp;
  if (dst == nullptr) return;  // uniform over the CTA
  {
    const int sy = tid % NS, q = tid / NS;
    float mx = 0.f;
#pragma unroll
    for (int i = 0; i < QV; ++i) {
      const float2 a = Cs[sy * PA_CLD + QV * q + i];
      mx = fmaxf(mx, fmaxf(fabsf(a.x), fabsf(a.y)));
    }
    red[q * NS + sy] = mx;
    __syncthreads();
    if (q == 0) {
      for (int qq = 1; qq < QN; ++qq) mx = fmaxf(mx, red[qq * NS + sy]);
      const int sh = tc_scale_shift(mx);
      s_scale[sy] = ldexpf(1.f, sh);
      if (b0 + sy < n) (right ? inv_sa : inv_sb)[b0 + sy - s0] = ldexpf(1.f, -sh);
    }
    __syncthreads();
  }
  if (right && nB > (int)(b0 - s0)) {
    // symmetric: B' column of system s (< nB) = D (row s of L21), its own scale
    __shared__ float2 s_d[64];
    __shared__ float s_tsc[64];
    // the pivots are the elimination's output: through L2 (the rows of A21 read before the
    // wait may have brought a line of the diagonal block into L1 before it was written)
    if (tid < 64) s_d[tid] = __ldcg(A + (j0 + tid) + (j0 + tid) * lda);
    __syncthreads();
    const int sy = tid % NS, q = tid / NS;
    float mx = 0.f;
#pragma unroll
    for (int i = 0; i < QV; ++i) {
      const float2 a = cmulx(Cs[sy * PA_CLD + QV * q + i], s_d[QV * q + i]);
      mx = fmaxf(mx, fmaxf(fabsf(a.x), fabsf(a.y)));
    }
    red[q * NS + sy] = mx;
    __syncthreads();
    if (q == 0) {
      for (int qq = 1; qq < QN; ++qq) mx = fmaxf(mx, red[qq * NS + sy]);
      const int sh = tc_scale_shift(mx);
      s_tsc[sy] = ldexpf(1.f, sh);
      if (b0 + sy - s0 < nB) inv_sb[b0 + sy - s0] = ldexpf(1.f, -sh);
    }
    __syncthreads();
    const int v0 = 4 * (lane & 15);
    for (int sp = 2 * warp; sp < NS; sp += 16) {
      const int s2 = sp + (lane >> 4);
      if (b0 + s2 - s0 < nB) {
        const float sc = s_tsc[s2];
        const float2* cr = Cs + s2 * PA_CLD + v0;
        __half2 hv[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const float2 a = cmulx(cr[i], s_d[v0 + i]);
          hv[i] = __floats2half2_rn(a.x * sc, a.y * sc);
        }
        *reinterpret_cast<uint4*>(Bp + (b0 + s2 - s0) * TRI + v0) = *reinterpret_cast<const uint4*>(hv);
      }
    }
  }
  // 16-byte stores: a lane converts 4 consecutive v of one system; right -- one system per
  // warp pass (lanes 0..15 row 2m, 16..31 row 2m+1: 512 contiguous bytes), left -- two
  // systems per pass (256 bytes each)
  const int v0 = 4 * (lane & 15);
  if (right) {
    for (int sy = warp; sy < NS; sy += 8) {
      if (b0 + sy >= n) break;
      const float sc = s_scale[sy];
      const float2* cr = Cs + sy * PA_CLD + v0;
      __half2 hv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const float2 a = cr[i];
        hv[i] = (lane < 16) ? __floats2half2_rn(a.x * sc, -a.y * sc) : __floats2half2_rn(a.y * sc, a.x * sc);
      }
      const int64_t m = b0 + sy - s0;
      *reinterpret_cast<uint4*>(Ap + (2 * m + (lane >> 4)) * TRI + v0) = *reinterpret_cast<const uint4*>(hv);
    }
  } else {
    for (int sp = 2 * warp; sp < NS; sp += 16) {
      const int sy = sp + (lane >> 4);
      if (b0 + sy < n) {
        const float sc = s_scale[sy];
        const float2* cr = Cs + sy * PA_CLD + v0;
        __half2 hv[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const float2 a = cr[i];
          hv[i] = __floats2half2_rn(a.x * sc, a.y * sc);
        }
        const int64_t m = b0 + sy - s0;
        *reinterpret_cast<uint4*>(Bp + m * TRI + v0) = *reinterpret_cast<const uint4*>(hv);
      }
    }
  }
}

// ---- symmetric factorisation helpers ---------------------------------------------------
// B (K x N, ld K) = D L^T with L = rows of the matrix (N x K at L, ld lda) and D the pivots on
// the diagonal at dg (stride lda + 1): the explicit operand of the CUDA-core fallback update
template <typename T>
__global__ void k_dlt(const T* L, const T* dg, int64_t lda, int K, int N, T* B) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= (int64_t)K * N) return;
  const int k = (int)(e % K), c = (int)(e / K);
  B[e] = cmulx(dg[(int64_t)k * (lda + 1)], L[c + (int64_t)k * lda]);
}

// U = D L^T above the 64 x 64 diagonal blocks: block (I, J), I < J, from the transposed block
// (J, I) of L and the pivots of rows 64 I..: U[i][j] = d_i L[j][i] (the diagonal blocks
// already hold U11 from k_lu_inv64)
// One CTA per block pair I < J (linear index J (J - 1) / 2 + I: no CTA on or below the diagonal).
template <typename T>
__global__ void __launch_bounds__(256) k_sym_upper(T* A, int64_t lda, int64_t n) {
  const int64_t L = blockIdx.x;
  int J = (int)((1.0f + sqrtf(1.0f + 8.0f * (float)L)) * 0.5f);
  while ((int64_t)J * (J - 1) / 2 > L) --J;
  while ((int64_t)(J + 1) * J / 2 <= L) ++J;
  const int I = (int)(L - (int64_t)J * (J - 1) / 2);
  __shared__ T t[64][65];
  __shared__ T d[64];
  const int64_t r0 = 64 * (int64_t)I, c0 = 64 * (int64_t)J;
  const int tid = threadIdx.x;
  if (tid < 64) d[tid] = r0 + tid < n ? A[(r0 + tid) * (lda + 1)] : T{0, 0};
  for (int e = tid; e < 64 * 64; e += 256) {
    const int j = e & 63, i = e >> 6;  // L[c0 + j][r0 + i], coalesced along j
    t[i][j] = (c0 + j < n && r0 + i < n) ? A[(c0 + j) + (r0 + i) * lda] : T{0, 0};
  }
  __syncthreads();
  for (int e = tid; e < 64 * 64; e += 256) {
    const int i = e & 63, j = e >> 6;  // U[r0 + i][c0 + j], coalesced along i
    if (r0 + i < n && c0 + j < n) A[(r0 + i) + (c0 + j) * lda] = cmulx(d[i], t[i][j]);
  }
}

// Lookahead of the symmetric factorisation: the diagonal block at p0 takes the previous
// panel's contribution just before its elimination, block -= L D L^T with L = A[p0.., p0-64..]
// (kb x 64, the block row the previous panel has just solved) and D that panel's pivots
// A[p0-64+k, p0-64+k].  Only the lower triangle with the diagonal (what the symmetric
// elimination reads), FP32 sums.  A thread owns a 4 x 4 tile; tiles above the diagonal idle.
constexpr int SDU_LD = 65;
size_t sym_diag_update_smem() { return (size_t)2 * 64 * SDU_LD * sizeof(float2); }
__global__ void __launch_bounds__(256) k_sym_diag_update(float2* A, int64_t lda, int64_t p0, int kb) {
  extern __shared__ __align__(16) unsigned char smraw[];
  float2* Ls = reinterpret_cast<float2*>(smraw);  // Ls[k LD + r] = L[r][k]
  float2* Ds = Ls + 64 * SDU_LD;                  // Ds[k LD + c] = d_k L[c][k]
  const int tid = threadIdx.x;
  const int64_t q0 = p0 - 64;
  for (int e = tid; e < 64 * 64; e += 256) {
    const int r = e & 63, k = e >> 6;  // column k of L, coalesced along r
    const float2 l = r < kb ? A[(p0 + r) + (q0 + k) * lda] : make_float2(0.f, 0.f);
    Ls[k * SDU_LD + r] = l;
    Ds[k * SDU_LD + r] = cmulx(A[(q0 + k) * (lda + 1)], l);
  }
  __syncthreads();
  const int tr = tid >> 4, tc = tid & 15;
  if (tc > tr) return;
  float2 acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = make_float2(0.f, 0.f);
#pragma unroll 4
  for (int k = 0; k < 64; ++k) {
    float2 a[4], b[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      a[i] = Ls[k * SDU_LD + 4 * tr + i];
      b[i] = Ds[k * SDU_LD + 4 * tc + i];
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) cfma(acc[i][j], a[i], b[j]);
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int r = 4 * tr + i, c = 4 * tc + j;
      if (r >= c && r < kb) {
        float2& x = A[(p0 + r) + (p0 + c) * lda];
        x = make_float2(x.x - acc[i][j].x, x.y - acc[i][j].y);
      }
    }
}

// sampled asymmetry: sums of |a_ij - a_ji|^2 and |a_ij|^2 + |a_ji|^2 over rows i = s p, columns
// j = s q < i (FP64 sums, atomically added)
template <typename T>
__global__ void k_asym_sample(const T* A, int64_t lda, int64_t n, int64_t s, double* out) {
  const int64_t np = (n + s - 1) / s;
  double dsum = 0, nsum = 0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < np * np; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = (e % np) * s, j = (e / np) * s;
    if (j >= i) continue;
    const T a = A[i + j * lda], b = A[j + i * lda];
    const double dr = (double)a.x - (double)b.x, di = (double)a.y - (double)b.y;
    dsum += dr * dr + di * di;
    nsum += (double)a.x * a.x + (double)a.y * a.y + (double)b.x * b.x + (double)b.y * b.y;
  }
  for (int o = 16; o > 0; o >>= 1) {
    dsum += __shfl_xor_sync(0xffffffffu, dsum, o);
    nsum += __shfl_xor_sync(0xffffffffu, nsum, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(out, dsum);
    atomicAdd(out + 1, nsum);
  }
}

// copy of the block-lower part of a c64 matrix: column j from row 64 floor(j / 64) down (what
// the symmetric factorisation reads; the rest of the copy is written at its end).  Two rows
// per thread (16-byte accesses when lda and ldf are even and the bases 16-byte aligned).
__global__ void __launch_bounds__(256) k_copy_lower_c64(int64_t n, const float2* A, int64_t lda, float2* F,
                                                       int64_t ldf, int vec) {
  // a CTA per column, two elements per thread and step (one 16-byte access when aligned)
  for (int64_t j = blockIdx.x; j < n; j += gridDim.x) {
    const float2* a = A + j * lda;
    float2* f = F + j * ldf;
    for (int64_t i = (j / 64) * 64 + 2 * threadIdx.x; i < n; i += 2 * 256) {
      if (vec && i + 1 < n) {
        *reinterpret_cast<float4*>(f + i) = __ldcs(reinterpret_cast<const float4*>(a + i));
      } else {
        f[i] = a[i];
        if (i + 1 < n) f[i + 1] = a[i + 1];
      }
    }
  }
}

// the same block-lower part from a c128 matrix, rounded to c64 by integer operations: a CTA
// per column (its rows from the first row of the column's diagonal block on), four streaming
// loads in flight per thread -- no CTA of the grid falls wholly above the diagonal
__global__ void __launch_bounds__(256) k_convert_lower_c128(int64_t n, const double2* A, int64_t lda, float2* F,
                                                           int64_t ldf) {
  auto cvt = [](double2 a) { return make_float2(fsplit::to_float_rn(a.x), fsplit::to_float_rn(a.y)); };
  for (int64_t j = blockIdx.x; j < n; j += gridDim.x) {
    const double2* a = A + j * lda;
    float2* f = F + j * ldf;
    int64_t i = (j / 64) * 64 + threadIdx.x;
    for (; i + 3 * 256 < n; i += 4 * 256) {
      double2 v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) v[u] = __ldcs(a + i + u * 256);
#pragma unroll
      for (int u = 0; u < 4; ++u) f[i + u * 256] = cvt(v[u]);
    }
    for (; i < n; i += 256) f[i] = cvt(__ldcs(a + i));
  }
}

// ---- C -= A B  (complex; C m x n, A m x k, B k x n; all column-major with ld) -------------
constexpr int GT = 64, GK = 8;
template <typename T, typename R>
__global__ void __launch_bounds__(256) k_gemm_sub(T* C, int64_t ldc, const T* Am, int64_t lda,
                                                  const T* Bm, int64_t ldb, int64_t m, int64_t n,
                                                  int k) {
  __shared__ R As[2][GK][GT + 1];
  __shared__ R Bs[2][GK][GT + 1];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int64_t bm = blockIdx.x * (int64_t)GT, bn = blockIdx.y * (int64_t)GT;
  R cr[4][4], ci[4][4];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) cr[i][j] = ci[i][j] = 0;
  for (int k0 = 0; k0 < k; k0 += GK) {
    // load A tile GT x GK and B tile GK x GT (256 threads, 2 elements each)
    for (int e = threadIdx.x; e < GT * GK; e += 256) {
      int r = e % GT, c = e / GT;
      int64_t gr = bm + r;
      int gc = k0 + c;
      T a = (gr < m && gc < k) ? Am[gr + gc * lda] : cmk<T>(0, 0);
      As[0][c][r] = a.x;
      As[1][c][r] = a.y;
      int rb = e % GK, cb = e / GK;
      int64_t gcol = bn + cb;
      int grow = k0 + rb;
      T b = (gcol < n && grow < k) ? Bm[grow + gcol * ldb] : cmk<T>(0, 0);
      Bs[0][rb][cb] = b.x;
      Bs[1][rb][cb] = b.y;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GK; ++kk) {
      R ar[4], ai[4], br[4], bi[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        ar[i] = As[0][kk][tx + 16 * i];
        ai[i] = As[1][kk][tx + 16 * i];
        br[i] = Bs[0][kk][ty + 16 * i];
        bi[i] = Bs[1][kk][ty + 16 * i];
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          cr[i][j] += ar[i] * br[j] - ai[i] * bi[j];
          ci[i][j] += ar[i] * bi[j] + ai[i] * br[j];
        }
    }
    __syncthreads();
  }
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      int64_t r = bm + tx + 16 * i, c = bn + ty + 16 * j;
      if (r < m && c < n) {
        T v = C[r + c * ldc];
        C[r + c * ldc] = cmk<T>(v.x - cr[i][j], v.y - ci[i][j]);
      }
    }
}

// ---- triangular solves on one right-hand side ------------------------------------------
// diagonal block solve by one CTA (rows [k0, k0+kb)); lower=1: unit lower, forward;
// lower=0: upper, backward
template <typename T>
__global__ void k_trsv_block(const T* A, int64_t lda, T* b, int64_t k0, int kb, int lower) {
  extern __shared__ unsigned char smraw[];
  T* D = reinterpret_cast<T*>(smraw);  // kb x kb diagonal block, column-major
  __shared__ double xr[128], xi[128];
  for (int e = threadIdx.x; e < kb * kb; e += blockDim.x) {
    int r = e % kb, c = e / kb;
    D[e] = A[(k0 + r) + (k0 + c) * lda];
  }
  for (int i = threadIdx.x; i < kb; i += blockDim.x) {
    xr[i] = b[k0 + i].x;
    xi[i] = b[k0 + i].y;
  }
  __syncthreads();
  if (lower) {
    for (int k = 0; k < kb; ++k) {
      double vr = xr[k], vi = xi[k];
      for (int i = k + 1 + threadIdx.x; i < kb; i += blockDim.x) {
        T l = D[i + k * kb];
        xr[i] -= l.x * vr - l.y * vi;
        xi[i] -= l.x * vi + l.y * vr;
      }
      __syncthreads();
    }
  } else {
    for (int k = kb - 1; k >= 0; --k) {
      if (threadIdx.x == 0) {
        T d = D[k + k * kb];
        double den = (double)d.x * d.x + (double)d.y * d.y;
        double r = (xr[k] * d.x + xi[k] * d.y) / den, im = (xi[k] * d.x - xr[k] * d.y) / den;
        xr[k] = r;
        xi[k] = im;
      }
      __syncthreads();
      double vr = xr[k], vi = xi[k];
      for (int i = threadIdx.x; i < k; i += blockDim.x) {
        T u = D[i + k * kb];
        xr[i] -= u.x * vr - u.y * vi;
        xi[i] -= u.x * vi + u.y * vr;
      }
      __syncthreads();
    }
  }
  for (int i = threadIdx.x; i < kb; i += blockDim.x) b[k0 + i] = cmk<T>(xr[i], xi[i]);
}

// b[rows] -= A[rows, k0:k0+kb] x[k0:k0+kb]  for rows in [r0, r1)
template <typename T>
__global__ void k_trsv_update(const T* A, int64_t lda, T* b, int64_t k0, int kb, int64_t r0,
                              int64_t r1) {
  int64_t i = r0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= r1) return;
  double sr = 0, si = 0;
  for (int k = 0; k < kb; ++k) {
    T a = A[i + (k0 + k) * lda];
    T x = b[k0 + k];
    sr += (double)a.x * x.x - (double)a.y * x.y;
    si += (double)a.x * x.y + (double)a.y * x.x;
  }
  T v = b[i];
  b[i] = cmk<T>(v.x - sr, v.y - si);
}

// ---- inverses of the 64 x 64 diagonal blocks of L (unit lower) and U (upper) ----------
// dinv + b * 2 * 4096: Linv_b then Uinv_b, column-major 64 x 64 (identity beyond rb)
template <typename T, typename RT>
__global__ void k_invert_diag(const T* A, int64_t lda, int64_t n, T* dinv) {
  extern __shared__ unsigned char smraw[];
  T* D = reinterpret_cast<T*>(smraw);   // 64 x 65 row-major
  T* X = D + 64 * 65;                   // 64 columns x 65 (column j of the inverse)
  const int b = blockIdx.x;
  const int64_t r0 = (int64_t)b * 64;
  const int rb = (int)(n - r0 < 64 ? n - r0 : 64);
  for (int e = threadIdx.x; e < 64 * 64; e += blockDim.x) {
    int i = e % 64, c = e / 64;
    T v;
    v.x = (RT)(i == c ? 1 : 0);
    v.y = 0;
    if (i < rb && c < rb) v = A[(r0 + i) + (r0 + c) * lda];
    D[i * 65 + c] = v;
  }
  __syncthreads();
  const int j = threadIdx.x;  // one column of each inverse per thread
  T* x = X + j * 65;
  T* Lout = dinv + (int64_t)b * 2 * 4096;
  T* Uout = Lout + 4096;
  // L x = e_j (unit lower)
  for (int i = 0; i < 64; ++i) {
    T v;
    v.x = (RT)(i == j ? 1 : 0);
    v.y = 0;
    if (i > j)
      for (int m = j; m < i; ++m) {
        T l = D[i * 65 + m], xm = x[m];
        v.x -= l.x * xm.x - l.y * xm.y;
        v.y -= l.x * xm.y + l.y * xm.x;
      }
    x[i] = v;
  }
  for (int i = 0; i < 64; ++i) Lout[j * 64 + i] = x[i];
  // U x = e_j (upper)
  for (int i = 63; i >= 0; --i) {
    T v;
    v.x = (RT)(i == j ? 1 : 0);
    v.y = 0;
    if (i < j)
      for (int m = i + 1; m <= j; ++m) {
        T u = D[i * 65 + m], xm = x[m];
        v.x -= u.x * xm.x - u.y * xm.y;
        v.y -= u.x * xm.y + u.y * xm.x;
      }
    if (i > j) {
      v.x = 0;
      v.y = 0;
    } else {
      T d = D[i * 65 + i];
      RT den = d.x * d.x + d.y * d.y;
      T q;
      q.x = (v.x * d.x + v.y * d.y) / den;
      q.y = (v.y * d.x - v.x * d.y) / den;
      v = q;
    }
    x[i] = v;
  }
  for (int i = 0; i < 64; ++i) Uout[j * 64 + i] = x[i];
}

// ---- triangular solve on one right-hand side as a wavefront ------------------------------
// Block rows of 64 are owned round-robin by co-resident CTAs (cooperative launch).  The
// solution is written to `out`, which starts filled with a sentinel (a NaN bit pattern that
// arithmetic does not produce), so a solved value is its own "ready" flag: a thread that
// needs block k spins (bounded) on exactly the 16 values it multiplies, with no counter, no
// fence and no block barrier inside the dependency walk.  The factor block of the next
// dependency and the thread's slice of the diagonal block's inverse are loaded ahead.  After
// the walk the CTA solves its diagonal block (inverse matvec) and stores its 64 values.
// lower = 1: unit lower, forward; lower = 0: upper, backward.  rhs: the right-hand side
// (read only).  Arithmetic in RT.  A wait that runs out sets status bit 8 and uses zeros.
constexpr unsigned long long SENT32 = 0x7FC0DEAD7FC0DEADull;  // two FP32 NaNs, payload 0xDEAD
constexpr unsigned long long SENT64 = 0x7FF8DEADBEEF0001ull;  // one FP64 NaN with a payload
constexpr long long TRSV_SPIN_MAX = 1LL << 22;

// a solved value as it is in memory (read from L2, never from a stale L1 line), and whether
// it is still the sentinel (for c128 each 8-byte half is checked: a 16-byte store may land
// in two parts)
__device__ __forceinline__ float2 ld_raw(const float2* p) {
  const unsigned long long u = *reinterpret_cast<const volatile unsigned long long*>(p);
  float2 v;
  v.x = __uint_as_float((unsigned)(u & 0xffffffffull));
  v.y = __uint_as_float((unsigned)(u >> 32));
  return v;
}
__device__ __forceinline__ double2 ld_raw(const double2* p) {
  const volatile unsigned long long* q = reinterpret_cast<const volatile unsigned long long*>(p);
  double2 v;
  v.x = __longlong_as_double((long long)q[0]);
  v.y = __longlong_as_double((long long)q[1]);
  return v;
}
__device__ __forceinline__ bool is_sent(float2 v) {
  return (((unsigned long long)__float_as_uint(v.y) << 32) | __float_as_uint(v.x)) == SENT32;
}
__device__ __forceinline__ bool is_sent(double2 v) {
  return (unsigned long long)__double_as_longlong(v.x) == SENT64 ||
         (unsigned long long)__double_as_longlong(v.y) == SENT64;
}

template <typename T>
__global__ void k_fill_sentinel(T* v, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned long long* u = reinterpret_cast<unsigned long long*>(v + i);
  if (sizeof(T) == 8) {
    u[0] = SENT32;
  } else {
    u[0] = SENT64;
    u[1] = SENT64;
  }
}

// ring of factor blocks for the wavefront solve: stages of 16 x 256 elements
template <typename T>
struct TrsvRing {
  static constexpr int STG = sizeof(T) == 8 ? 3 : 2;
  static constexpr size_t BYTES = (size_t)STG * 16 * 256 * sizeof(T);
};
// one element global -> shared, asynchronously (zero-filled when !in: nothing is read)
__device__ __forceinline__ void cp_async_el(float2* dst, const float2* src, bool in) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
               "l"(src), "r"(in ? 8 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_async_el(double2* dst, const double2* src, bool in) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
               "l"(src), "r"(in ? 16 : 0)
               : "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

template <typename T, typename RT>
__global__ void __launch_bounds__(256) k_trsv_wave(const T* A, int64_t lda, int64_t n, const T* rhs, T* out,
                                                   int lower, int* status, const T* dinv, long long spin_max) {
  constexpr int STG = TrsvRing<T>::STG;
  extern __shared__ __align__(16) unsigned char trsv_smraw[];
  T* ring = reinterpret_cast<T*>(trsv_smraw);  // STG x 16 x 256 elements
  __shared__ RT sr[64], si[64];
  __shared__ RT pr[4][64], pim[4][64];
  const int nblk = (int)((n + 63) / 64);
  const int tid = threadIdx.x, r = tid & 63, q = tid >> 6;
  const T zero = {0, 0};
  bool timed_out = false;
  for (int t = blockIdx.x; t < nblk; t += gridDim.x) {
    const int b = lower ? t : nblk - 1 - t;
    const int64_t r0 = (int64_t)b * 64;
    const int rb = (int)(n - r0 < 64 ? n - r0 : 64);
    // this thread's 16 entries of the diagonal block's inverse (row r, columns q*16..)
    const T* Di = dinv + (int64_t)b * 2 * 4096 + (lower ? 0 : 4096);
    T dv[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) dv[c] = Di[(q * 16 + c) * 64 + r];
    // the block's right-hand side, needed right after the last dependency
    const T bv = (tid < rb) ? rhs[r0 + tid] : zero;
    // this thread's 16 entries of the factor block of dependency s (row r0 + r) go into ring
    // stage s % TRSV_STG by cp.async: each thread reads back only what it copied itself, so
    // the walk needs no barrier
    auto issue_blk = [&](int s) {
      if (s < t) {
        const int k = lower ? s : nblk - 1 - s;
        const int64_t c0 = (int64_t)k * 64;
        const int cb = (int)(n - c0 < 64 ? n - c0 : 64);
        const T* Ar = A + (r0 + r) + c0 * lda;
        T* st = ring + (size_t)(s % STG) * 16 * 256;
#pragma unroll
        for (int c = 0; c < 16; ++c) {
          const int col = q * 16 + c;
          const bool in = r < rb && col < cb;
          cp_async_el(st + c * 256 + tid, in ? Ar + (int64_t)col * lda : A, in);
        }
      }
      asm volatile("cp.async.commit_group;" ::: "memory");
    };
    // the solved values of dependency s: lane l of a warp (all its lanes share q) reads value
    // q*16 + (l & 15) as it is in memory (maybe still the sentinel): the warp's 16 values
    // are one 128-byte line, so one request per warp per poll, and they are passed to every
    // lane with shuffles once all are written
    const int lane = tid & 31;
    auto load_x = [&](int s) -> T {
      const int k = lower ? s : nblk - 1 - s;
      const int c = q * 16 + (lane & 15);
      return c < (int)(n - (int64_t)k * 64) ? ld_raw(out + (int64_t)k * 64 + c) : zero;
    };
    RT ar = 0, ai = 0;
    T x1 = zero, x2 = zero;
#pragma unroll
    for (int j = 0; j < STG - 1; ++j) issue_blk(j);
    if (t > 0) x1 = load_x(0);
    if (t > 1) x2 = load_x(1);
    for (int s = 0; s < t; ++s) {
      issue_blk(s + STG - 1);
      // solved values two dependencies ahead are requested before this one is used
      T v = x1;
      x1 = x2;
      if (s + 2 < t) x2 = load_x(s + 2);
      cp_async_wait<STG - 1>();  // this thread's copies of dependency s have landed
      const T* st = ring + (size_t)(s % STG) * 16 * 256;
      T cur[16];
#pragma unroll
      for (int c = 0; c < 16; ++c) cur[c] = st[c * 256 + tid];
      long long it = 0;
      while (!__all_sync(0xffffffffu, !is_sent(v))) {  // warp-uniform
        if (++it > spin_max) {
          if (!timed_out) atomicOr(status, 8);
          timed_out = true;
          if (is_sent(v)) v = zero;
          break;
        }
        if (is_sent(v)) v = load_x(s);
      }
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        const T xc = shfl_c(v, c);
        ar += (RT)cur[c].x * (RT)xc.x - (RT)cur[c].y * (RT)xc.y;
        ai += (RT)cur[c].x * (RT)xc.y + (RT)cur[c].y * (RT)xc.x;
      }
    }
    cp_async_wait<0>();
    pr[q][r] = ar;
    pim[q][r] = ai;
    __syncthreads();
    if (tid < 64) {
      RT vr = 0, vi = 0;
      if (tid < rb) {
        vr = (RT)bv.x - (pr[0][tid] + pr[1][tid] + pr[2][tid] + pr[3][tid]);
        vi = (RT)bv.y - (pim[0][tid] + pim[1][tid] + pim[2][tid] + pim[3][tid]);
      }
      sr[tid] = vr;
      si[tid] = vi;
    }
    __syncthreads();
    // x_b = inv(D_b) * rhs_b  (64 x 64 matvec, 4 quarter sums per row)
    {
      RT accr = 0, acci = 0;
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        const T m = dv[c];
        accr += (RT)m.x * sr[q * 16 + c] - (RT)m.y * si[q * 16 + c];
        acci += (RT)m.x * si[q * 16 + c] + (RT)m.y * sr[q * 16 + c];
      }
      pr[q][r] = accr;
      pim[q][r] = acci;
    }
    __syncthreads();
    if (tid < rb) {
      T o;
      o.x = pr[0][tid] + pr[1][tid] + pr[2][tid] + pr[3][tid];
      o.y = pim[0][tid] + pim[1][tid] + pim[2][tid] + pim[3][tid];
      __stcg(out + r0 + tid, o);
    }
    __syncthreads();  // pr / pim are rewritten by the next block row
  }
}

// out[i] = in[perm[i]]: the row interchanges of the factorisation applied as one gather
template <typename T>
__global__ void k_permute(const T* in, T* out, const int* perm, int64_t n) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = in[perm[i]];
}

// ---- FP64 matvec y = alpha A x + beta y  (A c128 or c64) --------------------------------
constexpr int MV_SLABS = 32;
// x (complex FP64) split into float hi + lo parts: (re_hi, im_hi, re_lo, im_lo)
__global__ void k_split_x(int64_t n, const double* x, float4* xs) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double xr = x[2 * i], xi = x[2 * i + 1];
  float rh = (float)xr, ih = (float)xi;
  xs[i] = make_float4(rh, ih, (float)(xr - (double)rh), (float)(xi - (double)ih));
}

// s_hi + s_lo += p with the rounding error of the addition kept (TwoSum)
__device__ __forceinline__ void two_sum_acc(float& sh, float& sl, float p) {
  float s = __fadd_rn(sh, p);
  float bb = __fsub_rn(s, sh);
  float t = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  sh = s;
  sl = __fadd_rn(sl, t);
}

// partial sums of A x for a c64 matrix with FP64-level accuracy from FP32 arithmetic:
// each product a * x_hi is split exactly into p + e (e = fma(a, x_hi, -p)), p is added with
// TwoSum, e and a * x_lo go to the low part (compensated dot product of Ogita, Rump and
// Oishi, SIAM J. Sci. Comput. 26 (2005)).
__global__ void k_gemv_partial_c64_df(int64_t n, const float2* A, int64_t lda, const float4* xs,
                                      double* part) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int s = blockIdx.y;
  int64_t c0 = n * s / MV_SLABS, c1 = n * (s + 1) / MV_SLABS;
  if (i >= n) return;
  float shr = 0.f, slr = 0.f, shi = 0.f, sli = 0.f;
  for (int64_t j = c0; j < c1; ++j) {
    float2 a = A[i + j * lda];
    float4 xv = xs[j];
    float p, e;
    p = __fmul_rn(a.x, xv.x);
    e = fmaf(a.x, xv.x, -p);
    two_sum_acc(shr, slr, p);
    slr = __fadd_rn(slr, e);
    p = __fmul_rn(-a.y, xv.y);
    e = fmaf(-a.y, xv.y, -p);
    two_sum_acc(shr, slr, p);
    slr = __fadd_rn(slr, e);
    slr = __fadd_rn(slr, __fsub_rn(__fmul_rn(a.x, xv.z), __fmul_rn(a.y, xv.w)));
    p = __fmul_rn(a.x, xv.y);
    e = fmaf(a.x, xv.y, -p);
    two_sum_acc(shi, sli, p);
    sli = __fadd_rn(sli, e);
    p = __fmul_rn(a.y, xv.x);
    e = fmaf(a.y, xv.x, -p);
    two_sum_acc(shi, sli, p);
    sli = __fadd_rn(sli, e);
    sli = __fadd_rn(sli, __fadd_rn(__fmul_rn(a.x, xv.w), __fmul_rn(a.y, xv.z)));
  }
  part[2 * (s * n + i)] = (double)shr + (double)slr;
  part[2 * (s * n + i) + 1] = (double)shi + (double)sli;
}

// the same with two rows per thread: one 16-byte load brings a[i, j] and a[i+1, j] (even i,
// even lda), and the two rows are independent accumulation chains.  The real and imaginary
// parts of a row travel as the two lanes of packed FP32 operations (sm_100 FFMA2 / FADD2 /
// FMUL2, each lane rounded as its scalar counterpart):
//   (re, im) += (a_r, a_r) (x_r, x_i) + (a_i, a_i) (-x_i, x_r),
// every product kept exactly (TwoProduct: p and fma(a, x, -p)) and added to the high part with
// its rounding error (TwoSum); the low-part terms (x's low half) in plain FP32.
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {  // a - b, one rounding
  return __ffma2_rn(b, make_float2(-1.f, -1.f), a);
}
__device__ __forceinline__ void two_sum2(float2& sh, float2& sl, float2 p) {
  const float2 t = __fadd2_rn(sh, p);
  const float2 bb = sub2(t, sh);
  sl = __fadd2_rn(sl, __fadd2_rn(sub2(sh, sub2(t, bb)), sub2(p, bb)));
  sh = t;
}
__device__ __forceinline__ void cdf_acc2(float2 A, float2 B, float2 X1, float2 X2, float2 L1, float2 L2, float2& sh,
                                         float2& sl) {
  float2 p = __fmul2_rn(A, X1);
  float2 e = __ffma2_rn(A, X1, make_float2(-p.x, -p.y));
  two_sum2(sh, sl, p);
  sl = __fadd2_rn(sl, e);
  p = __fmul2_rn(B, X2);
  e = __ffma2_rn(B, X2, make_float2(-p.x, -p.y));
  two_sum2(sh, sl, p);
  sl = __fadd2_rn(sl, e);
  sl = __ffma2_rn(A, L1, sl);
  sl = __ffma2_rn(B, L2, sl);
}
__global__ void k_gemv_partial_c64_df2(int64_t n, const float2* A, int64_t lda, const float4* xs,
                                       double* part) {
  const int64_t i = 2 * (blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
  const int s = blockIdx.y;
  const int64_t c0 = n * s / MV_SLABS, c1 = n * (s + 1) / MV_SLABS;
  if (i >= n) return;
  const bool two = i + 1 < n;
  float2 h0 = make_float2(0.f, 0.f), l0 = h0, h1 = h0, l1 = h0;
#pragma unroll 4
  for (int64_t j = c0; j < c1; ++j) {
    const float4 xv = xs[j];
    const float2 X1 = make_float2(xv.x, xv.y), X2 = make_float2(-xv.y, xv.x);
    const float2 L1 = make_float2(xv.z, xv.w), L2 = make_float2(-xv.w, xv.z);
    float4 a;
    if (two) {
      a = *reinterpret_cast<const float4*>(A + i + j * lda);
    } else {
      const float2 a0 = A[i + j * lda];
      a = make_float4(a0.x, a0.y, 0.f, 0.f);
    }
    cdf_acc2(make_float2(a.x, a.x), make_float2(a.y, a.y), X1, X2, L1, L2, h0, l0);
    cdf_acc2(make_float2(a.z, a.z), make_float2(a.w, a.w), X1, X2, L1, L2, h1, l1);
  }
  part[2 * (s * n + i)] = (double)h0.x + (double)l0.x;
  part[2 * (s * n + i) + 1] = (double)h0.y + (double)l0.y;
  if (two) {
    part[2 * (s * n + i + 1)] = (double)h1.x + (double)l1.x;
    part[2 * (s * n + i + 1) + 1] = (double)h1.y + (double)l1.y;
  }
}

// partial sums of A x for a c128 matrix on the FP32 pipes: each entry split into hi + lo
// floats (fsplit.h), hi * x_hi kept exactly (TwoProduct) and added with TwoSum, the terms of
// the low parts (hi * x_lo, lo * x_hi) accumulated in FP32 -- the compensated dot product of
// k_gemv_partial_c64_df2 with the matrix's own low part added.  About 2^-47 relative per
// product, against a few FP64 multiply-adds per entry at GB300's FP64 rate.
__global__ void k_gemv_partial_c128_df(int64_t n, const double2* A, int64_t lda, const float4* xs,
                                       double* part) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int s = blockIdx.y;
  const int64_t c0 = n * s / MV_SLABS, c1 = n * (s + 1) / MV_SLABS;
  if (i >= n) return;
  float2 h = make_float2(0.f, 0.f), l = h;
  auto term = [&](const double2 a, const float4 xv) {
    const float2 X1 = make_float2(xv.x, xv.y), X2 = make_float2(-xv.y, xv.x);
    const float2 L1 = make_float2(xv.z, xv.w), L2 = make_float2(-xv.w, xv.z);
    float2 ar, ai;
    fsplit::split_f64(a.x, &ar.x, &ar.y);
    fsplit::split_f64(a.y, &ai.x, &ai.y);
    cdf_acc2(make_float2(ar.x, ar.x), make_float2(ai.x, ai.x), X1, X2, L1, L2, h, l);
    l = __ffma2_rn(make_float2(ar.y, ar.y), X1, l);
    l = __ffma2_rn(make_float2(ai.y, ai.y), X2, l);
  };
  // eight streaming loads in flight per thread before their arithmetic (the matrix is read
  // once per matvec; its latency, not the FP32 work, set the pace with four)
  const double2* Ai = A + i;
  int64_t j = c0;
  for (; j + 8 <= c1; j += 8) {
    double2 a[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) a[u] = __ldcs(Ai + (j + u) * lda);
#pragma unroll
    for (int u = 0; u < 8; ++u) term(a[u], xs[j + u]);
  }
  for (; j < c1; ++j) term(__ldcs(Ai + j * lda), xs[j]);
  part[2 * (s * n + i)] = (double)h.x + (double)l.x;
  part[2 * (s * n + i) + 1] = (double)h.y + (double)l.y;
}

__global__ void k_gemv_reduce(int64_t n, const double* part, double* y, double alpha, double beta) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double sr = 0, si = 0;
  for (int s = 0; s < MV_SLABS; ++s) {
    sr += part[2 * (s * n + i)];
    si += part[2 * (s * n + i) + 1];
  }
  double yr = beta == 0.0 ? 0.0 : beta * y[2 * i], yi = beta == 0.0 ? 0.0 : beta * y[2 * i + 1];
  y[2 * i] = alpha * sr + yr;
  y[2 * i + 1] = alpha * si + yi;
}

__global__ void k_c128_to_c64(int64_t rows, int64_t cols, const double* s, int64_t lds, float* d,
                              int64_t ldd) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int64_t c = blockIdx.y;
  for (; c < cols; c += gridDim.y)
    if (i < rows) {
      // rounded by integer operations: a conversion instruction runs on GB300's FP64 pipe
      d[2 * (i + c * ldd)] = fsplit::to_float_rn(s[2 * (i + c * lds)]);
      d[2 * (i + c * ldd) + 1] = fsplit::to_float_rn(s[2 * (i + c * lds) + 1]);
    }
}
__global__ void k_c64_to_c128(int64_t rows, int64_t cols, const float* s, int64_t lds, double* d,
                              int64_t ldd) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int64_t c = blockIdx.y;
  for (; c < cols; c += gridDim.y)
    if (i < rows) {
      d[2 * (i + c * ldd)] = fsplit::f2d(s[2 * (i + c * lds)]);
      d[2 * (i + c * ldd) + 1] = fsplit::f2d(s[2 * (i + c * lds) + 1]);
    }
}

__global__ void k_axpy(int64_t n, double ar, double ai, const double* x, double* y) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double xr = x[2 * i], xi = x[2 * i + 1];
  y[2 * i] += ar * xr - ai * xi;
  y[2 * i + 1] += ar * xi + ai * xr;
}

// deterministic sum of |x|^2: fixed grid, per-block partials, single-block final pass
__global__ void k_norm2_part(int64_t n, const double* x, double* part) {
  __shared__ double s[256];
  double acc = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    acc += x[2 * i] * x[2 * i] + x[2 * i + 1] * x[2 * i + 1];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}
__global__ void k_sum_part(int np, const double* part, double* out) {
  __shared__ double s[256];
  double acc = 0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) acc += part[i];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = s[0];
}

// h[k] = <V_k, w> (conjugated first argument), one block per k
__global__ void k_dots(int64_t n, const double* V, int64_t ldv, const double* w, double* h) {
  __shared__ double sr[256], si[256];
  int k = blockIdx.x;
  const double* v = V + 2 * (int64_t)k * ldv;
  double ar = 0, ai = 0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    double vr = v[2 * i], vi = v[2 * i + 1], wr = w[2 * i], wi = w[2 * i + 1];
    ar += vr * wr + vi * wi;
    ai += vr * wi - vi * wr;
  }
  sr[threadIdx.x] = ar;
  si[threadIdx.x] = ai;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      sr[threadIdx.x] += sr[threadIdx.x + o];
      si[threadIdx.x] += si[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    h[2 * k] = sr[0];
    h[2 * k + 1] = si[0];
  }
}
// w -= sum_k h_k V_k
__global__ void k_gemv_sub(int64_t n, int m, const double* V, int64_t ldv, const double* h, double* w) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double sr = 0, si = 0;
  for (int k = 0; k < m; ++k) {
    double vr = V[2 * (i + k * ldv)], vi = V[2 * (i + k * ldv) + 1];
    double hr = h[2 * k], hi = h[2 * k + 1];
    sr += hr * vr - hi * vi;
    si += hr * vi + hi * vr;
  }
  w[2 * i] -= sr;
  w[2 * i + 1] -= si;
}

template <typename T, typename R>
struct LUSteps {
  beast_ctx* ctx;
  T* A;
  int64_t lda, n;
  int* ipiv;
  cudaStream_t st;
  size_t tcwork_bytes;
  int laswp(int64_t c0, int64_t c1, int64_t p0, int64_t p1) {
    if (c1 <= c0 || p1 <= p0) return BEAST_OK;
    ProfScope ps(ctx, PK_LASWP, (double)(c1 - c0) * (p1 - p0) * 2 * sizeof(T));
    k_laswp<T><<<(unsigned)((c1 - c0 + 255) / 256), 256, 0, st>>>(A, lda, c0, c1, p0, p1, ipiv);
    BEAST_CUDA_TRY(ctx, cudaGetLastError());
    return BEAST_OK;
  }
  // U12 = L11^{-1} A12 for columns [c0, c1), L11 = the diagonal block at j0
  int trsm(int64_t j0, int kb, int64_t c0, int64_t c1) {
    if (c1 <= c0) return BEAST_OK;
    ProfScope ps(ctx, PK_TRSM, 4.0 * (double)(c1 - c0) * kb * kb);
    constexpr int NS = TrsmTile<T>::NS;
    k_trsm_tile<T, R, false><<<(unsigned)((c1 - c0 + NS - 1) / NS), TrsmTile<T>::NT, trsm_tile_smem<T>(), st>>>(
        A, lda, j0, kb, c0, c1);
    BEAST_CUDA_TRY(ctx, cudaGetLastError());
    return BEAST_OK;
  }
  // A[r0:r0+m, c0:c0+nc] -= A[r0:r0+m, k0:k0+k] A[k0:k0+k, c0:c0+nc]
  int gemm(int64_t r0, int64_t m, int64_t c0, int64_t nc, int64_t k0, int k, void* tcwork) {
    return gemm2(r0, m, c0, nc, 0, 0, k0, k, tcwork);
  }
  // the same on an L-shaped region: rows [r0, r0+m0) of columns [c0, c0+n0), then rows
  // [r0, r0+m1) (m1 <= m0) of the next n1 columns -- one tensor-core launch for both
  // whether gemm2 with these sizes runs (and on the tensor cores)
  static bool gemm2_runs(int64_t m0, int64_t n0, int64_t m1, int64_t n1, int k) {
    return m0 > 0 && k > 0 && (n0 > 0 || (m1 > 0 && n1 > 0));
  }
  bool gemm2_tc(int64_t m0, int64_t n0, int64_t n1, int k, const void* tcwork) const {
    return sizeof(T) == 8 && tcwork && m0 >= 64 && n0 + n1 >= 64 && k % 32 == 0;
  }
  // prepped: the FP16 operands are already in tcwork (k_panel_apply wrote them)
  int gemm2(int64_t r0, int64_t m0, int64_t c0, int64_t n0, int64_t m1, int64_t n1, int64_t k0, int k,
            void* tcwork, bool prepped = false) {
    if (!gemm2_runs(m0, n0, m1, n1, k)) return BEAST_OK;
    const bool tc = gemm2_tc(m0, n0, n1, k, tcwork);
    if (tc)  // brackets its operand preparation and its tensor-core launch separately
      return tc_gemm_sub(ctx, reinterpret_cast<float2*>(A), lda, r0, k0, c0, m0, n0, m1, n1, k, tcwork,
                         tcwork_bytes, prepped);
    ProfScope ps(ctx, PK_GEMM, 8.0 * (double)k * ((double)m0 * n0 + (double)m1 * n1));
    const int64_t ms[2] = {m0, m1}, cs[2] = {c0, c0 + n0}, ns[2] = {n0, n1};
    for (int r = 0; r < 2; ++r) {
      if (ms[r] <= 0 || ns[r] <= 0) continue;
      dim3 g((unsigned)((ms[r] + GT - 1) / GT), (unsigned)((ns[r] + GT - 1) / GT));
      k_gemm_sub<T, R><<<g, 256, 0, st>>>(A + r0 + cs[r] * lda, lda, A + r0 + k0 * lda, lda, A + k0 + cs[r] * lda,
                                          lda, ms[r], ns[r], k);
      BEAST_CUDA_TRY(ctx, cudaGetLastError());
    }
    return BEAST_OK;
  }
  // symmetric update: A[rowA.., rowB..] (m x nc) -= L1 D L2^T, L1 = A[rowA.., colA..],
  // L2 = A[rowB.., colA..], D the pivots on the diagonal at colA..; lower: only the tiles on or
  // below the diagonal (tensor cores; the CUDA-core fallback updates the whole rectangle)
  bool symgemm_tc(int64_t m, int64_t nc, int k, const void* tcwork) const {
    return sizeof(T) == 8 && tcwork && m >= 64 && nc >= 64 && k % 32 == 0;
  }
  // a_skip: the prepped operands were written for a_skip more rows above rowA
  int symgemm(int64_t rowA, int64_t m, int64_t rowB, int64_t nc, int64_t colA, int k, bool lower, void* tcwork,
              bool prepped = false, int64_t a_skip = 0) {
    if (m <= 0 || nc <= 0 || k <= 0) return BEAST_OK;
    const bool tc = symgemm_tc(m, nc, k, tcwork);
    if (tc)  // brackets its operand preparation and its tensor-core launch separately
      return tc_gemm_sym(ctx, reinterpret_cast<float2*>(A), lda, rowA, colA, rowB, m, nc, k, lower, tcwork,
                         tcwork_bytes, prepped, prepped ? a_skip : 0);
    ProfScope ps(ctx, PK_GEMM, 8.0 * (double)k * (double)m * nc);
    T* B = nullptr;
    BEAST_CUDA_TRY(ctx, cudaMallocAsync(&B, (size_t)k * nc * sizeof(T), st));
    const int64_t tot = (int64_t)k * nc;
    k_dlt<T><<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(A + rowB + colA * lda, A + colA + colA * lda, lda, k,
                                                            (int)nc, B);
    dim3 g((unsigned)((m + GT - 1) / GT), (unsigned)((nc + GT - 1) / GT));
    k_gemm_sub<T, R><<<g, 256, 0, st>>>(A + rowA + rowB * lda, lda, A + rowA + colA * lda, lda, B, k, m, nc, k);
    BEAST_CUDA_TRY(ctx, cudaGetLastError());
    BEAST_CUDA_TRY(ctx, cudaFreeAsync(B, st));
    return BEAST_OK;
  }
};

// Two-level right-looking LU: column blocks of NB are factored with nb-wide panels (panel,
// interchanges, TRSM and GEMM restricted to the block); then the block's interchanges are
// applied to the other columns and the trailing matrix gets one rank-NB update
// (TRSM for U12, GEMM with K = NB -- on the tensor cores for complex FP32).
//
// sym (unpivoted c64 with 64-wide panels; A near complex-symmetric, the factors serving as the
// preconditioner of a refined solve): an LDL^T-type factorisation that keeps only the lower
// triangle current -- the diagonal blocks are factored from their lower triangle mirrored,
// U12 = D L21^T is never formed in FP32 (the updates take it from L21 and the pivots), the
// in-block and mid-block updates cover only the rows below, the trailing update only the
// tiles on or below the diagonal: about half the work.  At the end U = D L^T is written above
// the diagonal blocks, so the factors have the layout of the LU.
template <typename T, typename R>
int lu_factor_t(beast_ctx* ctx, int64_t n, T* A, int64_t lda, int* ipiv, int* info, bool pivot, bool sym) {
  cudaStream_t st = ctx->stream;
  const int G0 = std::max(1, ctx->num_sms);
  const size_t smem_cap = 220 * 1024;
  // panel width: 64; with pivoting the cooperative panel kernel holds its share of the panel's
  // rows in shared memory, which narrows the panel for very tall matrices
  int nb = 64;
  const int64_t rows0 = (n + G0 - 1) / G0;
  if (pivot) {
    while (nb > 8 && (size_t)(rows0 * (nb + 1) + nb) * sizeof(T) > smem_cap) nb /= 2;
    if ((size_t)(rows0 * (nb + 1) + nb) * sizeof(T) > smem_cap)
      return beast_fail(ctx, BEAST_ERR_ARG, "matrix too large for the shared-memory panel");
  }
  // outer / mid block widths in columns: 16 and 4 panels (with pivoting a single level);
  // unpivoted, BEAST_LU_NB / BEAST_LU_NB2 override them (multiples of the panel width, the
  // mid width dividing the outer one, the outer one at most TC_SYM_KMAX)
  int NB = 16 * nb;
  int64_t NB2 = pivot ? NB : 4 * nb;
  if (!pivot) {
    const char* e1 = getenv("BEAST_LU_NB");
    const char* e2 = getenv("BEAST_LU_NB2");
    const int b1 = e1 ? atoi(e1) : NB, b2 = e2 ? atoi(e2) : (int)NB2;
    if (b2 >= nb && b2 % nb == 0 && b1 >= b2 && b1 % b2 == 0 && b1 <= TC_SYM_KMAX) {
      NB = b1;
      NB2 = b2;
    }
  }
  const size_t panel_smem = (size_t)(rows0 * (nb + 1) + nb) * sizeof(T);
  if (pivot)
    BEAST_CUDA_TRY(ctx, cudaFuncSetAttribute(k_panel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)panel_smem));
  // unpivoted c64 with 64-wide panels: k_lu_inv64 also inverts the block's triangles and
  // k_panel_apply does both triangular solves (and the FP16 operands of the in-block update)
  const bool apply_path = !pivot && sizeof(T) == 8 && nb == TRI;
  sym = sym && apply_path;
  const size_t getrf_sm = (size_t)TRI * (TRI + 1) * sizeof(T);
  BEAST_CUDA_TRY(ctx, cudaFuncSetAttribute(k_getrf64<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)getrf_sm));
  BEAST_CUDA_TRY(ctx, cudaFuncSetAttribute(k_lu_inv64<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)getrf_sm));
  BEAST_CUDA_TRY(ctx, cudaFuncSetAttribute(k_lu_inv64<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)getrf_sm));
  BEAST_CUDA_TRY(ctx, cudaFuncSetAttribute(k_lu_inv64<T, false, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)getrf_sm));
  BEAST_CUDA_TRY(ctx, cudaFuncSetAttribute(k_lu_inv64<T, true, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)getrf_sm));
  BEAST_CUDA_TRY(ctx, cudaFuncSetAttribute(k_lu_inv64<T, false, 2, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)getrf_sm));
  BEAST_CUDA_TRY(ctx, cudaFuncSetAttribute(k_lu_inv64<T, true, 2, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)getrf_sm));
  // the diagonal-block elimination with 2 x 2 tiles on 1024 threads (default), 2 x 4 tiles on 512
  // (BEAST_LU_DIAG_TILE=24) or 4 x 4 tiles on 256 (BEAST_LU_DIAG_TILE=4): the same arithmetic
  // per element, different thread counts
  const char* dt_env = getenv("BEAST_LU_DIAG_TILE");
  const int dtile = dt_env && dt_env[0] == '4' ? 44 : (dt_env && dt_env[0] == '2' && dt_env[1] == '4' ? 24 : 22);
  if (apply_path)
    BEAST_CUDA_TRY(ctx, cudaFuncSetAttribute(k_panel_apply<64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)panel_apply_smem()));
    BEAST_CUDA_TRY(ctx, cudaFuncSetAttribute(k_panel_apply<32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)panel_apply_smem()));
  BEAST_CUDA_TRY(ctx, cudaFuncSetAttribute(k_trsm_tile<T, R, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)trsm_tile_smem<T>()));
  BEAST_CUDA_TRY(ctx, cudaFuncSetAttribute(k_trsm_tile<T, R, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)trsm_tile_smem<T>()));
  if (pivot) {
    int occ = 0;
    BEAST_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_panel<T>, 256, panel_smem));
    if (occ < 1) return beast_fail(ctx, BEAST_ERR_CUDA, "panel kernel does not fit on an SM");
  }
  size_t need = 2 * G0 * sizeof(double) + 2 * G0 * sizeof(int) + (2 * (size_t)G0 * nb + 2 * nb) * sizeof(T) +
                8 * sizeof(unsigned int) + 256;
  char* scr = nullptr;
  BEAST_CUDA_TRY(ctx, cudaMallocAsync(&scr, need, st));
  double* cval = reinterpret_cast<double*>(scr);
  int* cidx = reinterpret_cast<int*>(cval + 2 * G0);
  T* crow = reinterpret_cast<T*>(((uintptr_t)(cidx + 2 * G0) + 15) & ~(uintptr_t)15);
  T* rowj = crow + 2 * (size_t)G0 * nb;
  unsigned int* bar = reinterpret_cast<unsigned int*>(rowj + 2 * nb);
  int* dinfo = reinterpret_cast<int*>(bar + 4);
  auto diag = [&](bool sy, int64_t jd, int kd, T* out_inv, cudaStream_t s_) {
    if (dtile == 22 && sy)
      k_lu_inv64<T, true, 2><<<1, TRI * TRI / 4, getrf_sm, s_>>>(A, lda, jd, kd, dinfo, out_inv);
    else if (dtile == 22)
      k_lu_inv64<T, false, 2><<<1, TRI * TRI / 4, getrf_sm, s_>>>(A, lda, jd, kd, dinfo, out_inv);
    else if (dtile == 24 && sy)
      k_lu_inv64<T, true, 2, 4><<<1, TRI * TRI / 8, getrf_sm, s_>>>(A, lda, jd, kd, dinfo, out_inv);
    else if (dtile == 24)
      k_lu_inv64<T, false, 2, 4><<<1, TRI * TRI / 8, getrf_sm, s_>>>(A, lda, jd, kd, dinfo, out_inv);
    else if (sy)
      k_lu_inv64<T, true><<<1, 256, getrf_sm, s_>>>(A, lda, jd, kd, dinfo, out_inv);
    else
      k_lu_inv64<T, false><<<1, 256, getrf_sm, s_>>>(A, lda, jd, kd, dinfo, out_inv);
  };
  BEAST_CUDA_TRY(ctx, cudaMemsetAsync(bar, 0, 4 * sizeof(unsigned int) + sizeof(int), st));
  BEAST_CUDA_TRY(ctx, cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), st));
  GridSync gs{bar, bar + 1, reinterpret_cast<int*>(bar + 2)};
  // tensor-core workspace: the FP16 operands of the largest update (M, N <= n, K <= NB)
  void* tcwork = nullptr;
  size_t tcwork_bytes = 0;
  if (sizeof(T) == 8 && tc_gemm_supported(A, lda, NB) && n > NB) {
    tcwork_bytes = tc_gemm_work_bytes(n, n, NB);
    BEAST_CUDA_TRY(ctx, cudaMallocAsync(&tcwork, tcwork_bytes, st));
  }
  LUSteps<T, R> S{ctx, A, lda, n, ipiv, st, tcwork_bytes};
  // lookahead (symmetric path with tensor-core updates; BEAST_LU_LOOKAHEAD=1): while a panel's
  // other rows and its update run on the context's stream, the second stream solves the next
  // panel's block row, updates and eliminates the next diagonal block.  ahead: this panel's
  // elimination has run there (event la_ev[lu_par]).
  const char* la_env = getenv("BEAST_LU_LOOKAHEAD");
  const bool la = sym && tcwork && la_env && la_env[0] == '1' && ctx_lookahead_streams(ctx);
  if (la)
    BEAST_CUDA_TRY(ctx, cudaFuncSetAttribute(k_sym_diag_update, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)sym_diag_update_smem()));
  bool ahead = false;
  int lu_par = 0;

  int rc = BEAST_OK;
  // unpivoted, the outer block is factored in mid blocks of NB2 columns: the panels update
  // only their mid block (and its rows beyond it), the mid block updates the rest of the
  // outer block with K = NB2, and the outer block the trailing matrix with K = NB -- fewer
  // passes of narrow (K = nb) updates over the same columns
  for (int64_t J0 = 0; J0 < n && rc == BEAST_OK; J0 += NB) {
    const int64_t J1 = std::min<int64_t>(n, J0 + NB);
    for (int64_t M0 = J0; M0 < J1 && rc == BEAST_OK; M0 += NB2) {
    const int64_t M1 = std::min<int64_t>(J1, M0 + NB2);
    for (int64_t j0 = M0; j0 < M1 && rc == BEAST_OK; j0 += nb) {
      int kb = (int)std::min<int64_t>(nb, M1 - j0);
      int64_t M = n - j0;
      int rows_per = (int)((M + G0 - 1) / G0);
      int G = (int)((M + rows_per - 1) / rows_per);
      size_t sm = (size_t)(rows_per * (kb + 1) + kb) * sizeof(T);
      if (pivot) {
        void* args[] = {&A, &lda, &n, &j0, &kb, &rows_per, &ipiv, &dinfo, &cval, &cidx, &crow, &rowj, &gs};
        {
          ProfScope ps(ctx, PK_PANEL, 8.0 * (double)M * kb * kb / 2);
          BEAST_CUDA_TRY(ctx, cudaLaunchCooperativeKernel((void*)k_panel<T>, G, 256, args, sm, st));
        }
        // interchanges inside the column block
        if ((rc = S.laswp(J0, j0, j0, j0 + kb))) break;
        if ((rc = S.laswp(j0 + kb, J1, j0, j0 + kb))) break;
      }
      // the in-block update (all rows below, mid-block columns) and, unpivoted, the mid
      // block's rows of the columns beyond it, as one L-shaped update
      const int64_t u_m0 = n - j0 - kb, u_n0 = M1 - j0 - kb, u_m1 = pivot ? 0 : M1 - j0 - kb,
                    u_n1 = pivot ? 0 : n - M1;
      bool applied = false, prepped = false;
      // lookahead for this panel: a full next panel inside the mid block with rows below it
      const bool next = la && kb == TRI && j0 + 2 * TRI <= M1 && n - j0 - kb > TRI;
      const int64_t skip = next ? TRI : 0;  // rows of the in-block update left to the second stream
      if (!pivot) {
        // no pivoting: diagonal block LU, then L21 = A21 U11^{-1} for every row below
        ProfScope ps(ctx, PK_PANEL, 8.0 * (double)M * kb * kb / 2, 0);
        constexpr int NS = TrsmTile<T>::NS;
        const int64_t rb = n - j0 - kb;
        T* dblk = apply_path ? reinterpret_cast<T*>(lu_dinv(ipiv, n)) + (j0 / TRI) * 2 * TRI * TRI : nullptr;
        ctx->launches += ahead ? 0 : 1;
        if (ahead)
          BEAST_CUDA_TRY(ctx, cudaStreamWaitEvent(st, ctx->la_ev[lu_par], 0));
        else if (apply_path)
          diag(sym, j0, kb, dblk, st);
        else
          k_getrf64<T><<<1, 256, getrf_sm, st>>>(A, lda, j0, kb, dinfo);
        if (apply_path && kb == TRI && rb > 0) {
          // L21 and U12 (every column to the right: no later interchange touches these rows)
          // in one launch, with the FP16 operands of the update below when it runs on the
          // tensor cores
          // (symmetric: L21 only, and the update is rows below x the rest of the mid block)
          const int64_t nBs = sym ? u_n0 : 0;
          prepped = sym ? (nBs > 0 && S.symgemm_tc(u_m0 - skip, nBs, kb, tcwork))
                        : (S.gemm2_runs(u_m0, u_n0, u_m1, u_n1, kb) && S.gemm2_tc(u_m0, u_n0, u_n1, kb, tcwork));
          void *Apv = nullptr, *Bpv = nullptr;
          float *isa = nullptr, *isb = nullptr;
          if (prepped) tc_gemm_operands(tcwork, u_m0, sym ? nBs : u_n0 + u_n1, kb, &Apv, &isa, &Bpv, &isb);
          const int nR = (int)((rb + 63) / 64);
          float2* Af = reinterpret_cast<float2*>(A);
          const float2* inv = reinterpret_cast<const float2*>(dblk);
          const int nBp = prepped ? (int)nBs : 0;
          if (next) {
            // second stream: block row j0 + 64 (its L rows and operands), then the next diagonal
            // block's update and elimination; it has to see this panel's elimination and the
            // previous in-block update (both on it, or both here)
            cudaStream_t ax = ctx->aux;
            if (ahead) {
              BEAST_CUDA_TRY(ctx, cudaStreamWaitEvent(ax, ctx->la_ev[3], 0));
            } else {
              BEAST_CUDA_TRY(ctx, cudaEventRecord(ctx->la_ev[4], st));
              BEAST_CUDA_TRY(ctx, cudaStreamWaitEvent(ax, ctx->la_ev[4], 0));
            }
            k_panel_apply<64><<<1, 256, panel_apply_smem(), ax>>>(Af, lda, j0, n, inv, nR, static_cast<__half2*>(Apv),
                                                              isa, static_cast<__half2*>(Bpv), isb, nBp, 0);
            BEAST_CUDA_TRY(ctx, cudaEventRecord(ctx->la_ev[2], ax));
            k_sym_diag_update<<<1, 256, sym_diag_update_smem(), ax>>>(Af, lda, j0 + TRI, TRI);
            diag(true, j0 + TRI, TRI, dblk + 2 * TRI * TRI, ax);
            lu_par ^= 1;
            BEAST_CUDA_TRY(ctx, cudaEventRecord(ctx->la_ev[lu_par], ax));
            ctx->launches += 3;
            // here: the other block rows, then (after the second stream's operands) the update
            if (nR > 1) {
              k_panel_apply<64><<<(unsigned)(nR - 1), 256, panel_apply_smem(), st>>>(
                  Af, lda, j0, n, inv, nR, static_cast<__half2*>(Apv), isa, static_cast<__half2*>(Bpv), isb, nBp, 1);
              ctx->launches += 1;
            }
            BEAST_CUDA_TRY(ctx, cudaStreamWaitEvent(st, ctx->la_ev[2], 0));
          } else {
            // 32 systems per CTA: twice the CTAs of half the work, so that more warps hide the
            // shared-memory latency of the triangular products
            const int nR32 = (int)((rb + 31) / 32);
            // a programmatic dependent launch: its CTAs take the SMs the one-CTA elimination
            // leaves idle and load their rows while it runs
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3((unsigned)(sym ? nR32 : 2 * nR32));
            cfg.blockDim = dim3(256);
            cfg.dynamicSmemBytes = panel_apply_smem();
            cfg.stream = st;
            cudaLaunchAttribute pdl[1];
            pdl[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
            pdl[0].val.programmaticStreamSerializationAllowed = 1;
            cfg.attrs = pdl;
            cfg.numAttrs = 1;
            BEAST_CUDA_TRY(ctx, cudaLaunchKernelEx(&cfg, k_panel_apply<32>, Af, lda, j0, n, inv, nR32,
                                                   static_cast<__half2*>(Apv), isa, static_cast<__half2*>(Bpv), isb,
                                                   nBp, 0));
            ctx->launches += 1;
          }
          applied = true;
        } else if (rb > 0) {
          k_trsm_tile<T, R, true><<<(unsigned)((rb + NS - 1) / NS), TrsmTile<T>::NT, trsm_tile_smem<T>(), st>>>(
              A, lda, j0, kb, j0 + kb, n);
          ctx->launches += 1;
        }
        BEAST_CUDA_TRY(ctx, cudaGetLastError());
      }
      // TRSM + GEMM for the rest of the block.  Unpivoted, no later interchange touches
      // these rows, so U12 of this panel is solved for every column to its right at once and
      // the block's rows of the columns beyond the block are updated here too (what the
      // pivoted path does per panel after the block).
      if (sym) {
        // with the next panel's elimination running on the second stream, the update's
        // persistent grid leaves two SMs to it (a CTA of the update needs a whole SM: one held
        // by the elimination would hold back the update's tiles until it ends)
        ctx->tc_sm_reserve = next ? 2 : 0;
        rc = S.symgemm(j0 + kb + skip, u_m0 - skip, j0 + kb, u_n0, j0, kb, false, tcwork, prepped, skip);
        ctx->tc_sm_reserve = 0;
        if (rc) break;
        if (next) BEAST_CUDA_TRY(ctx, cudaEventRecord(ctx->la_ev[3], st));
        ahead = next;
        continue;
      }
      if (!applied && (rc = S.trsm(j0, kb, j0 + kb, pivot ? J1 : n))) break;
      if ((rc = S.gemm2(j0 + kb, u_m0, j0 + kb, u_n0, u_m1, u_n1, j0, kb, tcwork, prepped))) break;
    }
    if (rc) break;
    // mid-block update: rows below x the rest of the outer block, and the rest of the outer
    // block's rows x the columns beyond it (K = NB2; nothing when pivoting: NB2 = NB)
    if (M1 < J1) {
      rc = sym ? S.symgemm(M1, n - M1, M1, J1 - M1, M0, (int)(M1 - M0), false, tcwork)
               : S.gemm2(M1, n - M1, M1, J1 - M1, J1 - M1, n - J1, M0, (int)(M1 - M0), tcwork);
      if (rc) break;
    }
    }
    if (rc) break;
    // the block's interchanges on the columns left and right of it
    if (pivot) {
      if ((rc = S.laswp(0, J0, J0, J1))) break;
      if ((rc = S.laswp(J1, n, J0, J1))) break;
    }
    if (J1 < n && sym) {
      rc = S.symgemm(J1, n - J1, J1, n - J1, J0, (int)(J1 - J0), true, tcwork);
    } else if (J1 < n) {
      // U12 = L11^{-1} A12 (blocked: nb-row TRSM, then GEMM on the rows below inside the
      // block); done per panel above when unpivoted
      for (int64_t j0 = J0; pivot && j0 < J1 && rc == BEAST_OK; j0 += nb) {
        int kb = (int)std::min<int64_t>(nb, J1 - j0);
        if ((rc = S.trsm(j0, kb, J1, n))) break;
        if ((rc = S.gemm(j0 + kb, J1 - j0 - kb, J1, n - J1, j0, kb, tcwork))) break;
      }
      if (rc) break;
      // trailing update with K = NB
      rc = S.gemm(J1, n - J1, J1, n - J1, J0, (int)(J1 - J0), tcwork);
    }
  }
  if (la) {  // nothing of the second stream outlives the factorisation
    BEAST_CUDA_TRY(ctx, cudaEventRecord(ctx->la_ev[4], ctx->aux));
    BEAST_CUDA_TRY(ctx, cudaStreamWaitEvent(st, ctx->la_ev[4], 0));
  }
  if (tcwork) cudaFreeAsync(tcwork, st);
  int hinfo[3] = {0, 0, 0};
  BEAST_CUDA_TRY(ctx, cudaMemcpyAsync(&hinfo[0], dinfo, sizeof(int), cudaMemcpyDeviceToHost, st));
  BEAST_CUDA_TRY(ctx, cudaMemcpyAsync(&hinfo[1], bar + 2, sizeof(int), cudaMemcpyDeviceToHost, st));
  BEAST_CUDA_TRY(ctx, cudaMemcpyAsync(&hinfo[2], ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, st));
  BEAST_CUDA_TRY(ctx, cudaStreamSynchronize(st));
  BEAST_CUDA_TRY(ctx, cudaFreeAsync(scr, st));
  if (rc) return rc;
  if (hinfo[1]) return beast_fail(ctx, BEAST_ERR_TIMEOUT, "LU panel: grid barrier timed out");
  if (hinfo[2] & 4) return beast_fail(ctx, BEAST_ERR_TIMEOUT, "LU tensor-core update: wait timed out");
  *info = hinfo[0];
  // the sequential interchanges ipiv[0..n) as one permutation: perm[i] = source row of row i
  std::vector<int> hp(n), perm(n);
  for (int64_t i = 0; i < n; ++i) perm[i] = (int)i;
  if (pivot) {
    BEAST_CUDA_TRY(ctx, cudaMemcpy(hp.data(), ipiv, n * sizeof(int), cudaMemcpyDeviceToHost));
    for (int64_t k = 0; k < n; ++k) std::swap(perm[k], perm[hp[k]]);
  } else {
    BEAST_CUDA_TRY(ctx, cudaMemcpy(ipiv, perm.data(), n * sizeof(int), cudaMemcpyHostToDevice));
  }
  BEAST_CUDA_TRY(ctx, cudaMemcpy(ipiv + n, perm.data(), n * sizeof(int), cudaMemcpyHostToDevice));
  if (sym) {  // U = D L^T above the diagonal blocks
    const int64_t nbk = (n + 63) / 64;
    ProfScope ps(ctx, PK_CONVERT, (double)n * n * sizeof(T));
    if (nbk > 1) k_sym_upper<T><<<(unsigned)(nbk * (nbk - 1) / 2), 256, 0, st>>>(A, lda, n);
    BEAST_CUDA_TRY(ctx, cudaGetLastError());
  }
  // inverses of the diagonal blocks for the triangular solves (already written by k_lu_inv64
  // on the apply path)
  if (apply_path) return BEAST_OK;
  const size_t ism = (size_t)2 * 64 * 65 * sizeof(T);
  BEAST_CUDA_TRY(ctx, cudaFuncSetAttribute(k_invert_diag<T, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ism));
  k_invert_diag<T, R><<<(unsigned)((n + 63) / 64), 64, ism, st>>>(A, lda, n, reinterpret_cast<T*>(lu_dinv(ipiv, n)));
  BEAST_CUDA_TRY(ctx, cudaGetLastError());
  return BEAST_OK;
}

// P b -> forward sweep -> backward sweep, per right-hand side: tmp (n values) is the
// permuted right-hand side, then the backward sweep's output, copied back into b
template <typename T, typename RT>
int trsv_pair(beast_ctx* ctx, int64_t n, const T* A, int64_t lda, const int* perm, T* B, int64_t ldb,
              int64_t nrhs, T* tmp, const T* dinv) {
  cudaStream_t st = ctx->stream;
  const int nblk = (int)((n + 63) / 64);
  const size_t ring = TrsvRing<T>::BYTES;
  BEAST_CUDA_TRY(ctx, cudaFuncSetAttribute(k_trsv_wave<T, RT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ring));
  int occ = 0;
  BEAST_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_trsv_wave<T, RT>, 256, ring));
  const int G = std::max(1, std::min(nblk, ctx->num_sms * std::max(occ, 1)));
  int* status = ctx->d_flag;
  long long spin_max = ctx->trsv_spin_max > 0 ? ctx->trsv_spin_max : TRSV_SPIN_MAX;
  const unsigned ge = (unsigned)((n + 255) / 256);
  // a stale status from an earlier call must not be reported for this one
  BEAST_CUDA_TRY(ctx, cudaMemsetAsync(status, 0, sizeof(int), st));
  for (int64_t rr = 0; rr < nrhs; ++rr) {
    T* b = B + rr * ldb;
    // the two triangular solves read the factors once: n^2 elements
    ProfScope ps(ctx, PK_TRSV, (double)n * n * sizeof(T), 5);
    k_permute<T><<<ge, 256, 0, st>>>(b, tmp, perm, n);
    k_fill_sentinel<T><<<ge, 256, 0, st>>>(b, n);
    int lower = 1;
    const T* in = tmp;
    T* outp = b;
    void* args[] = {&A, &lda, &n, &in, &outp, &lower, &status, &dinv, &spin_max};
    BEAST_CUDA_TRY(ctx, cudaLaunchCooperativeKernel((void*)k_trsv_wave<T, RT>, G, 256, args, ring, st));
    k_fill_sentinel<T><<<ge, 256, 0, st>>>(tmp, n);
    lower = 0;
    in = b;
    outp = tmp;
    BEAST_CUDA_TRY(ctx, cudaLaunchCooperativeKernel((void*)k_trsv_wave<T, RT>, G, 256, args, ring, st));
    BEAST_CUDA_TRY(ctx, cudaMemcpyAsync(b, tmp, (size_t)n * sizeof(T), cudaMemcpyDeviceToDevice, st));
  }
  BEAST_CUDA_TRY(ctx, cudaGetLastError());
  return BEAST_OK;
}

template <typename T, typename RT>
int lu_solve_t(beast_ctx* ctx, int64_t n, const T* A, int64_t lda, const int* perm, T* B,
               int64_t ldb, int64_t nrhs, const T* dinv) {
  cudaStream_t st = ctx->stream;
  T* tmp = nullptr;
  BEAST_CUDA_TRY(ctx, cudaMallocAsync(&tmp, (size_t)n * sizeof(T), st));
  int rc = trsv_pair<T, RT>(ctx, n, A, lda, perm, B, ldb, nrhs, tmp, dinv);
  BEAST_CUDA_TRY(ctx, cudaFreeAsync(tmp, st));
  return rc;
}

// ---- allocation-free triangular solve ----------------------------------------------------
// Scratch of beast_lu_solve_noalloc: one right-hand side of up to NOALLOC_MAX_N complex128
// values (the permuted right-hand side, then the backward sweep's output).
// Held by every GPU that loads the library, for the life of the process.
constexpr int64_t NOALLOC_MAX_N = 65536;
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_MAX_N * 16];

template <typename T, typename RT>
int lu_solve_fixed_scratch(beast_ctx* ctx, int64_t n, const T* A, int64_t lda, const int* perm, T* B,
                           int64_t ldb, int64_t nrhs, unsigned char* scratch, const T* dinv) {
  // the scratch keeps the previous call's values; every value it is read for is written
  // first in this call (the permutation, then the sentinel fill)
  return trsv_pair<T, RT>(ctx, n, A, lda, perm, B, ldb, nrhs, reinterpret_cast<T*>(scratch), dinv);
}

}  // namespace

int lu_factor_dev(beast_ctx* ctx, int64_t n, void* A, int64_t lda, int dtype, int* ipiv, int* info,
                  bool pivot, bool sym) {
  if (dtype == BEAST_C64) return lu_factor_t<float2, float>(ctx, n, (float2*)A, lda, ipiv, info, pivot, sym);
  return lu_factor_t<double2, double>(ctx, n, (double2*)A, lda, ipiv, info, pivot, false);
}

double asym_sample(beast_ctx* ctx, int64_t n, const void* A, int64_t lda, int dtype) {
  if (n < 2) return 0.0;
  const int64_t s = std::max<int64_t>(1, n / 1400);  // about 10^6 pairs
  double* d = nullptr;
  if (cudaMallocAsync(&d, 2 * sizeof(double), ctx->stream) != cudaSuccess) return 1.0;
  cudaMemsetAsync(d, 0, 2 * sizeof(double), ctx->stream);
  if (dtype == BEAST_C64)
    k_asym_sample<float2><<<1024, 256, 0, ctx->stream>>>((const float2*)A, lda, n, s, d);
  else
    k_asym_sample<double2><<<1024, 256, 0, ctx->stream>>>((const double2*)A, lda, n, s, d);
  double h[2] = {0, 0};
  cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream);
  cudaFreeAsync(d, ctx->stream);
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return 1.0;
  return h[1] > 0 ? std::sqrt(2.0 * h[0] / h[1]) : 0.0;
}

// ipiv holds 2n ints: the pivots, then the permutation built by lu_factor_dev
int lu_solve_dev(beast_ctx* ctx, int64_t n, const void* A, int64_t lda, int dtype, const int* ipiv,
                 void* B, int64_t ldb, int64_t nrhs) {
  if (dtype == BEAST_C64)
    return lu_solve_t<float2, float>(ctx, n, (const float2*)A, lda, ipiv + n, (float2*)B, ldb, nrhs,
                                     (const float2*)lu_dinv(ipiv, n));
  return lu_solve_t<double2, double>(ctx, n, (const double2*)A, lda, ipiv + n, (double2*)B, ldb, nrhs,
                                     (const double2*)lu_dinv(ipiv, n));
}

// waits for the context stream and reports a triangular-solve flag wait that ran out (status
// bit 8, cleared at the start of every solve by trsv_pair)
int trsv_check(beast_ctx* ctx) {
  BEAST_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  int status = 0;
  BEAST_CUDA_TRY(ctx, cudaMemcpy(&status, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost));
  if (status & 8) return beast_fail(ctx, BEAST_ERR_TIMEOUT, "triangular solve: flag wait timed out");
  return BEAST_OK;
}

// scratch per call from the device's stream-ordered pool (cheap once the pool holds memory;
// nothing shared between contexts, streams or devices)
cudaError_t gemv_dev(int64_t n, const void* A, int64_t lda, int a_c64, const double* x, double* y,
                     double alpha, double beta, cudaStream_t st) {
  const size_t need = (size_t)MV_SLABS * n * 2 * sizeof(double) + (size_t)n * sizeof(float4) + 256;
  double* part = nullptr;
  cudaError_t e = cudaMallocAsync(&part, need, st);
  if (e != cudaSuccess) return e;
  dim3 g((unsigned)((n + 127) / 128), MV_SLABS);
  float4* xs = reinterpret_cast<float4*>(part + (size_t)MV_SLABS * n * 2);
  k_split_x<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, x, xs);
  if (a_c64) {
    if (lda % 2 == 0 && (reinterpret_cast<uintptr_t>(A) & 15) == 0) {
      dim3 g2((unsigned)((n + 255) / 256), MV_SLABS);
      k_gemv_partial_c64_df2<<<g2, 128, 0, st>>>(n, (const float2*)A, lda, xs, part);
    } else {
      k_gemv_partial_c64_df<<<g, 128, 0, st>>>(n, (const float2*)A, lda, xs, part);
    }
  } else
    k_gemv_partial_c128_df<<<g, 128, 0, st>>>(n, (const double2*)A, lda, xs, part);
  k_gemv_reduce<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, part, y, alpha, beta);
  e = cudaGetLastError();
  cudaFreeAsync(part, st);
  return e;
}

cudaError_t copy_lower_c64(int64_t n, const void* A, int64_t lda, void* F, int64_t ldf, cudaStream_t st) {
  const int vec = (lda % 2 == 0 && ldf % 2 == 0 && (reinterpret_cast<uintptr_t>(A) & 15) == 0 &&
                   (reinterpret_cast<uintptr_t>(F) & 15) == 0)
                      ? 1
                      : 0;
  if (n <= 0) return cudaSuccess;
  k_copy_lower_c64<<<(unsigned)std::min<int64_t>(n, 65535), 256, 0, st>>>(n, (const float2*)A, lda, (float2*)F, ldf,
                                                                          vec);
  return cudaGetLastError();
}

cudaError_t convert_lower_c128_to_c64(int64_t n, const void* A, int64_t lda, void* F, int64_t ldf, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_convert_lower_c128<<<(unsigned)std::min<int64_t>(n, 65535), 256, 0, st>>>(n, (const double2*)A, lda, (float2*)F,
                                                                              ldf);
  return cudaGetLastError();
}
cudaError_t convert_c128_to_c64(int64_t rows, int64_t cols, const double* src, int64_t lds, float* dst,
                                int64_t ldd, cudaStream_t st) {
  dim3 g((unsigned)((rows + 255) / 256), (unsigned)std::min<int64_t>(cols, 65535));
  k_c128_to_c64<<<g, 256, 0, st>>>(rows, cols, src, lds, dst, ldd);
  return cudaGetLastError();
}
cudaError_t convert_c64_to_c128(int64_t rows, int64_t cols, const float* src, int64_t lds, double* dst,
                                int64_t ldd, cudaStream_t st) {
  dim3 g((unsigned)((rows + 255) / 256), (unsigned)std::min<int64_t>(cols, 65535));
  k_c64_to_c128<<<g, 256, 0, st>>>(rows, cols, src, lds, dst, ldd);
  return cudaGetLastError();
}
cudaError_t vec_axpy(int64_t n, double ar, double ai, const double* x, double* y, cudaStream_t st) {
  k_axpy<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, ar, ai, x, y);
  return cudaGetLastError();
}
cudaError_t vec_copy(int64_t n, const double* x, double* y, cudaStream_t st) {
  return cudaMemcpyAsync(y, x, (size_t)n * 2 * sizeof(double), cudaMemcpyDeviceToDevice, st);
}
cudaError_t vec_norm2(int64_t n, const double* x, double* out, cudaStream_t st) {
  double* npart = nullptr;
  cudaError_t e = cudaMallocAsync(&npart, 256 * sizeof(double), st);
  if (e != cudaSuccess) return e;
  k_norm2_part<<<256, 256, 0, st>>>(n, x, npart);
  k_sum_part<<<1, 256, 0, st>>>(256, npart, out);
  e = cudaGetLastError();
  cudaFreeAsync(npart, st);
  return e;
}
cudaError_t vec_dots(int64_t n, int m, const double* V, int64_t ldv, const double* w, double* h,
                     cudaStream_t st) {
  if (m <= 0) return cudaSuccess;
  k_dots<<<m, 256, 0, st>>>(n, V, ldv, w, h);
  return cudaGetLastError();
}
cudaError_t vec_gemv_sub(int64_t n, int m, const double* V, int64_t ldv, const double* h, double* w,
                         cudaStream_t st) {
  if (m <= 0) return cudaSuccess;
  k_gemv_sub<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, m, V, ldv, h, w);
  return cudaGetLastError();
}

// Device address of the fixed scratch, looked up once per device with that device current.
// (In host code the array's name is only a host-side stand-in, never a device address.)
static unsigned char* noalloc_scratch(beast_ctx* ctx) {
  static std::mutex mtx;
  static unsigned char* addr[64] = {nullptr};
  std::lock_guard<std::mutex> lk(mtx);
  if (ctx->device < 0 || ctx->device >= 64) return nullptr;
  if (!addr[ctx->device]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess) return nullptr;
    addr[ctx->device] = static_cast<unsigned char*>(p);
  }
  return addr[ctx->device];
}

extern "C" int beast_lu_solve_noalloc(beast_ctx* ctx, const beast_lu* lu, int64_t nrhs, void* B,
                                      int64_t ldb) {
  if (!ctx) return BEAST_ERR_ARG;
  if (!lu || !B || nrhs < 0 || ldb < lu->n)
    return beast_fail(ctx, BEAST_ERR_ARG, "invalid solve arguments");
  if (lu->n > NOALLOC_MAX_N)
    return beast_fail(ctx, BEAST_ERR_ARG,
                      "beast_lu_solve_noalloc: n = " + std::to_string(lu->n) +
                          " exceeds the fixed scratch limit of " + std::to_string(NOALLOC_MAX_N) +
                          " unknowns; use beast_lu_solve");
  BEAST_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  unsigned char* scratch = noalloc_scratch(ctx);
  if (!scratch) return beast_fail(ctx, BEAST_ERR_CUDA, "cudaGetSymbolAddress of the fixed scratch failed");
  int rc;
  if (lu->dtype == BEAST_C64)
    rc = lu_solve_fixed_scratch<float2, float>(ctx, lu->n, (const float2*)lu->A, lu->lda, lu->ipiv + lu->n,
                                               (float2*)B, ldb, nrhs, scratch,
                                               (const float2*)lu_dinv(lu->ipiv, lu->n));
  else
    rc = lu_solve_fixed_scratch<double2, double>(ctx, lu->n, (const double2*)lu->A, lu->lda,
                                                 lu->ipiv + lu->n, (double2*)B, ldb, nrhs, scratch,
                                                 (const double2*)lu_dinv(lu->ipiv, lu->n));
  if (rc) return rc;
  return trsv_check(ctx);
}
