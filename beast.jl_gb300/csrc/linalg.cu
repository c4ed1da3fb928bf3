// linalg.cu -- dense complex LU with partial pivoting, triangular solves, FP64 matvec.
//
// Replaces LAPACK zgetrf/zgetrs behind `\` (src/solvers/lusolver.jl:30, src/solvers/lu.jl:40-47)
// for a device-resident matrix.  Right-looking blocked LU:
//   k_panel    cooperative kernel over the column panel: per column a grid-wide pivot
//              search (max |re|+|im|, first index on ties -- the izamax rule), the row swap
//              and the rank-1 update, with bounded-spin grid barriers (a barrier that gives
//              up sets a status word and the kernel returns; nothing hangs)
//   k_laswp    the panel's row interchanges applied to the other columns
//   k_trsm     U12 = L11^{-1} A12
//   k_gemm     A22 -= L21 U12 (complex, tiled through shared memory)
// The element type is complex FP64 (c128) or complex FP32 (c64).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.h"

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
template <typename T>
__global__ void k_panel(T* A, int64_t lda, int64_t n, int64_t j0, int nb, int* ipiv, int* info,
                        double* cand_val, int* cand_idx, GridSync gs) {
  const unsigned nblk = gridDim.x;
  const int64_t M = n - j0;
  const int64_t per = (M + nblk - 1) / nblk;
  const int64_t r0 = j0 + blockIdx.x * per, r1 = min(n, r0 + per);
  __shared__ double sval[256];
  __shared__ int sidx[256];
  __shared__ int piv_s;
  for (int jj = 0; jj < nb; ++jj) {
    const int64_t j = j0 + jj;
    // 1. local pivot candidate over own rows >= j
    double bv = -1.0;
    int bi = 0x7fffffff;
    for (int64_t i = max(r0, j) + threadIdx.x; i < r1; i += blockDim.x) {
      double v = cabs1(__ldcg(A + i + j * lda));
      if (v > bv || (v == bv && i < bi)) {
        bv = v;
        bi = (int)i;
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
    if (threadIdx.x == 0) {
      cand_val[blockIdx.x] = sval[0];
      cand_idx[blockIdx.x] = sidx[0];
    }
    if (!grid_barrier(gs, nblk)) return;
    // 2. global pivot (every CTA computes the same answer); CTA 0 swaps the panel rows
    if (threadIdx.x == 0) {
      double v = -1.0;
      int p = 0x7fffffff;
      for (unsigned b = 0; b < nblk; ++b) {
        double cv = ((volatile double*)cand_val)[b];
        int ci = ((volatile int*)cand_idx)[b];
        if (cv > v || (cv == v && ci < p)) {
          v = cv;
          p = ci;
        }
      }
      if (v <= 0.0) p = (int)j;
      piv_s = p;
      if (blockIdx.x == 0) {
        ipiv[j] = p;
        if (v <= 0.0 && *info == 0) *info = (int)j + 1;
      }
    }
    __syncthreads();
    const int64_t p = piv_s;
    if (blockIdx.x == 0 && p != j) {
      for (int k = threadIdx.x; k < nb; k += blockDim.x) {
        T a = __ldcg(A + j + (j0 + k) * lda);
        A[j + (j0 + k) * lda] = __ldcg(A + p + (j0 + k) * lda);
        A[p + (j0 + k) * lda] = a;
      }
    }
    if (!grid_barrier(gs, nblk)) return;
    // 3. scale column j below the diagonal and rank-1 update of the panel (own rows)
    T piv = __ldcg(A + j + j * lda);
    double den = (double)piv.x * piv.x + (double)piv.y * piv.y;
    if (den == 0.0) continue;
    double ir = piv.x / den, ii = -piv.y / den;
    for (int64_t i = max(r0, j + 1) + threadIdx.x; i < r1; i += blockDim.x) {
      T a = __ldcg(A + i + j * lda);
      double lr = a.x * ir - a.y * ii, li = a.x * ii + a.y * ir;
      A[i + j * lda] = cmk<T>(lr, li);
      for (int k = jj + 1; k < nb; ++k) {
        T u = __ldcg(A + j + (j0 + k) * lda);
        T c = __ldcg(A + i + (j0 + k) * lda);
        A[i + (j0 + k) * lda] = cmk<T>(c.x - (lr * u.x - li * u.y), c.y - (lr * u.y + li * u.x));
      }
    }
  }
}

// ---- row interchanges on columns outside the panel --------------------------------------
template <typename T>
__global__ void k_laswp(T* A, int64_t lda, int64_t ncols_total, int64_t j0, int nb, const int* ipiv) {
  int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  // columns [0, j0) and [j0+nb, n)
  int64_t col = c < j0 ? c : c + nb;
  if (col >= ncols_total) return;
  for (int k = 0; k < nb; ++k) {
    int64_t r = j0 + k, p = ipiv[j0 + k];
    if (p != r) {
      T a = A[r + col * lda];
      A[r + col * lda] = A[p + col * lda];
      A[p + col * lda] = a;
    }
  }
}

// ---- U12 = L11^{-1} A12 (unit lower), one thread per column -----------------------------
template <typename T>
__global__ void k_trsm(T* A, int64_t lda, int64_t n, int64_t j0, int nb) {
  extern __shared__ unsigned char smraw[];
  T* L = reinterpret_cast<T*>(smraw);  // nb x nb
  for (int k = threadIdx.x; k < nb * nb; k += blockDim.x) {
    int r = k % nb, c = k / nb;
    L[k] = A[(j0 + r) + (j0 + c) * lda];
  }
  __syncthreads();
  int64_t col = j0 + nb + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (col >= n) return;
  T* b = A + j0 + col * lda;
  for (int k = 0; k < nb; ++k) {
    T bk = b[k];
    for (int i = k + 1; i < nb; ++i) {
      T l = L[i + k * nb];
      T bi = b[i];
      b[i] = cmk<T>(bi.x - (l.x * bk.x - l.y * bk.y), bi.y - (l.x * bk.y + l.y * bk.x));
    }
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
  __shared__ double xr[128], xi[128];
  for (int i = threadIdx.x; i < kb; i += blockDim.x) {
    xr[i] = b[k0 + i].x;
    xi[i] = b[k0 + i].y;
  }
  __syncthreads();
  if (lower) {
    for (int k = 0; k < kb; ++k) {
      double vr = xr[k], vi = xi[k];
      for (int i = k + 1 + threadIdx.x; i < kb; i += blockDim.x) {
        T l = A[(k0 + i) + (k0 + k) * lda];
        xr[i] -= l.x * vr - l.y * vi;
        xi[i] -= l.x * vi + l.y * vr;
      }
      __syncthreads();
    }
  } else {
    for (int k = kb - 1; k >= 0; --k) {
      if (threadIdx.x == 0) {
        T d = A[(k0 + k) + (k0 + k) * lda];
        double den = (double)d.x * d.x + (double)d.y * d.y;
        double r = (xr[k] * d.x + xi[k] * d.y) / den, im = (xi[k] * d.x - xr[k] * d.y) / den;
        xr[k] = r;
        xi[k] = im;
      }
      __syncthreads();
      double vr = xr[k], vi = xi[k];
      for (int i = threadIdx.x; i < k; i += blockDim.x) {
        T u = A[(k0 + i) + (k0 + k) * lda];
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

// out[i] = in[perm[i]]: the row interchanges of the factorisation applied as one gather
template <typename T>
__global__ void k_permute(const T* in, T* out, const int* perm, int64_t n) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = in[perm[i]];
}

// ---- FP64 matvec y = alpha A x + beta y  (A c128 or c64) --------------------------------
constexpr int MV_SLABS = 32;
template <typename T>
__global__ void k_gemv_partial(int64_t n, const T* A, int64_t lda, const double* x, double* part) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int s = blockIdx.y;
  int64_t c0 = n * s / MV_SLABS, c1 = n * (s + 1) / MV_SLABS;
  if (i >= n) return;
  double sr = 0, si = 0;
  for (int64_t j = c0; j < c1; ++j) {
    T a = A[i + j * lda];
    double xr = x[2 * j], xi = x[2 * j + 1];
    sr += (double)a.x * xr - (double)a.y * xi;
    si += (double)a.x * xi + (double)a.y * xr;
  }
  part[2 * (s * n + i)] = sr;
  part[2 * (s * n + i) + 1] = si;
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
      d[2 * (i + c * ldd)] = (float)s[2 * (i + c * lds)];
      d[2 * (i + c * ldd) + 1] = (float)s[2 * (i + c * lds) + 1];
    }
}
__global__ void k_c64_to_c128(int64_t rows, int64_t cols, const float* s, int64_t lds, double* d,
                              int64_t ldd) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int64_t c = blockIdx.y;
  for (; c < cols; c += gridDim.y)
    if (i < rows) {
      d[2 * (i + c * ldd)] = s[2 * (i + c * lds)];
      d[2 * (i + c * ldd) + 1] = s[2 * (i + c * lds) + 1];
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
int lu_factor_t(beast_ctx* ctx, int64_t n, T* A, int64_t lda, int* ipiv, int* info) {
  cudaStream_t st = ctx->stream;
  const int nb = 64;
  // scratch for the panel kernel: candidates + barrier words + info
  const int maxblk = 1024;
  size_t need = maxblk * sizeof(double) + maxblk * sizeof(int) + 4 * sizeof(unsigned int) + sizeof(int);
  char* scr = nullptr;
  BEAST_CUDA_TRY(ctx, cudaMallocAsync(&scr, need, st));
  double* cval = reinterpret_cast<double*>(scr);
  int* cidx = reinterpret_cast<int*>(scr + maxblk * sizeof(double));
  unsigned int* bar = reinterpret_cast<unsigned int*>(scr + maxblk * (sizeof(double) + sizeof(int)));
  int* dinfo = reinterpret_cast<int*>(bar + 4);
  BEAST_CUDA_TRY(ctx, cudaMemsetAsync(bar, 0, 4 * sizeof(unsigned int) + sizeof(int), st));
  GridSync gs{bar, bar + 1, reinterpret_cast<int*>(bar + 2)};
  int occ = 0;
  BEAST_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_panel<T>, 256, 0));
  BEAST_CUDA_TRY(ctx, cudaFuncSetAttribute(k_trsm<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)(nb * nb * sizeof(T))));
  int rc = BEAST_OK;
  for (int64_t j0 = 0; j0 < n; j0 += nb) {
    int kb = (int)std::min<int64_t>(nb, n - j0);
    int64_t M = n - j0;
    int nblk = (int)std::min<int64_t>({(int64_t)ctx->num_sms * std::max(occ, 1), (M + 255) / 256, (int64_t)maxblk});
    nblk = std::max(nblk, 1);
    void* args[] = {&A, &lda, &n, &j0, &kb, &ipiv, &dinfo, &cval, &cidx, &gs};
    {
      ProfScope ps(ctx, PK_PANEL, 8.0 * (double)M * kb * kb / 2);
      BEAST_CUDA_TRY(ctx, cudaLaunchCooperativeKernel((void*)k_panel<T>, nblk, 256, args, 0, st));
    }
    int64_t other = n - kb;
    if (other > 0) {
      ProfScope ps(ctx, PK_LASWP, (double)other * kb * 2 * sizeof(T));
      k_laswp<T><<<(unsigned)((other + 255) / 256), 256, 0, st>>>(A, lda, n, j0, kb, ipiv);
    }
    int64_t rest = n - j0 - kb;
    if (rest > 0) {
      size_t smb = (size_t)kb * kb * sizeof(T);
      {
        ProfScope ps(ctx, PK_TRSM, 4.0 * (double)rest * kb * kb);
        k_trsm<T><<<(unsigned)((rest + 127) / 128), 128, smb, st>>>(A, lda, n, j0, kb);
      }
      dim3 g((unsigned)((rest + GT - 1) / GT), (unsigned)((rest + GT - 1) / GT));
      ProfScope ps(ctx, PK_GEMM, 8.0 * (double)rest * rest * kb);
      k_gemm_sub<T, R><<<g, 256, 0, st>>>(A + (j0 + kb) + (j0 + kb) * lda, lda, A + (j0 + kb) + j0 * lda,
                                          lda, A + j0 + (j0 + kb) * lda, lda, rest, rest, kb);
    }
    BEAST_CUDA_TRY(ctx, cudaGetLastError());
  }
  int hinfo[2] = {0, 0};
  BEAST_CUDA_TRY(ctx, cudaMemcpyAsync(&hinfo[0], dinfo, sizeof(int), cudaMemcpyDeviceToHost, st));
  BEAST_CUDA_TRY(ctx, cudaMemcpyAsync(&hinfo[1], bar + 2, sizeof(int), cudaMemcpyDeviceToHost, st));
  BEAST_CUDA_TRY(ctx, cudaStreamSynchronize(st));
  BEAST_CUDA_TRY(ctx, cudaFreeAsync(scr, st));
  if (hinfo[1]) return beast_fail(ctx, BEAST_ERR_TIMEOUT, "LU panel: grid barrier timed out");
  *info = hinfo[0];
  // the sequential interchanges ipiv[0..n) as one permutation: perm[i] = source row of row i
  std::vector<int> hp(n), perm(n);
  BEAST_CUDA_TRY(ctx, cudaMemcpy(hp.data(), ipiv, n * sizeof(int), cudaMemcpyDeviceToHost));
  for (int64_t i = 0; i < n; ++i) perm[i] = (int)i;
  for (int64_t k = 0; k < n; ++k) std::swap(perm[k], perm[hp[k]]);
  BEAST_CUDA_TRY(ctx, cudaMemcpy(ipiv + n, perm.data(), n * sizeof(int), cudaMemcpyHostToDevice));
  return rc;
}

template <typename T>
int lu_solve_t(beast_ctx* ctx, int64_t n, const T* A, int64_t lda, const int* perm, T* B,
               int64_t ldb, int64_t nrhs) {
  cudaStream_t st = ctx->stream;
  const int nb = 64;
  T* tmp = nullptr;
  BEAST_CUDA_TRY(ctx, cudaMallocAsync(&tmp, (size_t)n * sizeof(T), st));
  for (int64_t r = 0; r < nrhs; ++r) {
    T* b = B + r * ldb;
    BEAST_CUDA_TRY(ctx, cudaMemcpyAsync(tmp, b, (size_t)n * sizeof(T), cudaMemcpyDeviceToDevice, st));
    // the two triangular solves read the factors once: n^2 elements
    ProfScope ps(ctx, PK_TRSV, (double)n * n * sizeof(T), 1 + 4 * (int)((n + nb - 1) / nb));
    k_permute<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(tmp, b, perm, n);
    for (int64_t k0 = 0; k0 < n; k0 += nb) {
      int kb = (int)std::min<int64_t>(nb, n - k0);
      k_trsv_block<T><<<1, 128, 0, st>>>(A, lda, b, k0, kb, 1);
      int64_t r0 = k0 + kb;
      if (r0 < n) k_trsv_update<T><<<(unsigned)((n - r0 + 255) / 256), 256, 0, st>>>(A, lda, b, k0, kb, r0, n);
    }
    for (int64_t k0 = ((n - 1) / nb) * nb; k0 >= 0; k0 -= nb) {
      int kb = (int)std::min<int64_t>(nb, n - k0);
      k_trsv_block<T><<<1, 128, 0, st>>>(A, lda, b, k0, kb, 0);
      if (k0 > 0) k_trsv_update<T><<<(unsigned)((k0 + 255) / 256), 256, 0, st>>>(A, lda, b, k0, kb, 0, k0);
    }
  }
  BEAST_CUDA_TRY(ctx, cudaGetLastError());
  BEAST_CUDA_TRY(ctx, cudaFreeAsync(tmp, st));
  return BEAST_OK;
}

}  // namespace

int lu_factor_dev(beast_ctx* ctx, int64_t n, void* A, int64_t lda, int dtype, int* ipiv, int* info) {
  if (dtype == BEAST_C64) return lu_factor_t<float2, float>(ctx, n, (float2*)A, lda, ipiv, info);
  return lu_factor_t<double2, double>(ctx, n, (double2*)A, lda, ipiv, info);
}

// ipiv holds 2n ints: the pivots, then the permutation built by lu_factor_dev
int lu_solve_dev(beast_ctx* ctx, int64_t n, const void* A, int64_t lda, int dtype, const int* ipiv,
                 void* B, int64_t ldb, int64_t nrhs) {
  if (dtype == BEAST_C64)
    return lu_solve_t<float2>(ctx, n, (const float2*)A, lda, ipiv + n, (float2*)B, ldb, nrhs);
  return lu_solve_t<double2>(ctx, n, (const double2*)A, lda, ipiv + n, (double2*)B, ldb, nrhs);
}

static double* g_part = nullptr;
static size_t g_part_size = 0;

cudaError_t gemv_dev(int64_t n, const void* A, int64_t lda, int a_c64, const double* x, double* y,
                     double alpha, double beta, cudaStream_t st) {
  size_t need = (size_t)MV_SLABS * n * 2 * sizeof(double);
  if (need > g_part_size) {
    if (g_part) cudaFree(g_part);
    cudaError_t e = cudaMalloc(&g_part, need);
    if (e != cudaSuccess) {
      g_part = nullptr;
      g_part_size = 0;
      return e;
    }
    g_part_size = need;
  }
  dim3 g((unsigned)((n + 127) / 128), MV_SLABS);
  if (a_c64)
    k_gemv_partial<float2><<<g, 128, 0, st>>>(n, (const float2*)A, lda, x, g_part);
  else
    k_gemv_partial<double2><<<g, 128, 0, st>>>(n, (const double2*)A, lda, x, g_part);
  k_gemv_reduce<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, g_part, y, alpha, beta);
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
static double* g_npart = nullptr;
cudaError_t vec_norm2(int64_t n, const double* x, double* out, cudaStream_t st) {
  if (!g_npart) {
    cudaError_t e = cudaMalloc(&g_npart, 256 * sizeof(double));
    if (e != cudaSuccess) return e;
  }
  k_norm2_part<<<256, 256, 0, st>>>(n, x, g_npart);
  k_sum_part<<<1, 256, 0, st>>>(256, g_npart, out);
  return cudaGetLastError();
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
