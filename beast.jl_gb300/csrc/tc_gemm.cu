// tc_gemm.cu -- tensor-core (tcgen05, FP16 operands, FP32 accumulation) trailing update of
// the complex FP32 LU.
//
//   C -= A B   with C (M x N), A (M x K), B (K x N) complex64, column-major
//
// is evaluated as one real GEMM on the interleaved (re, im) storage:
//   C' (2M x N) -= A' (2M x 2K) B' (2K x N)
//   C'  = the real view of C (no copy: element (r, c) of the complex matrix occupies rows
//         2r, 2r+1 of column c of the real view)
//   A'  = A expanded into 2x2 real blocks [[ar, -ai], [ai, ar]], K-major, row pair of complex
//         row m scaled by a power of two s_m (expand_h)
//   B'  = the real view of B, column j scaled by a power of two t_j (convert_bh; both in
//         one launch, k_prep_h)
// Both operands are rounded to FP16 (11 significant bits, the precision of TF32) after the
// scaling puts each row's / column's largest magnitude in [2^13, 2^14), so the FP16 range
// never clips; the products accumulate in FP32 in TMEM and the epilogue multiplies by the
// exact factor 1 / (s_m t_j).  FP16 runs the tensor cores at twice the TF32 rate with half
// the operand bytes.
// Kernel k_tc_gemm: persistent CTAs over 128 x 256 tiles of C'; a single thread issues the
// TMA loads (128-byte swizzle, 4-stage ring over K) and the tcgen05.mma instructions (M=128,
// N=256, K=16 per instruction) into a 256-column TMEM accumulator; four epilogue warps read
// their 32 TMEM lanes with tcgen05.ld and apply C' -= D / (s t) as TMA reduce-adds of
// shared-memory chunks (C' is read and written by the TMA unit only).
// Every mbarrier wait is bounded by a clock budget: on expiry the CTA raises a status bit,
// still frees its TMEM and returns (the host turns the bit into BEAST_ERR_TIMEOUT).
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "internal.h"
#include "tc_tiles.h"

namespace {

constexpr int TM = TC_TM, TN = TC_TN, TK = 64;  // tile M (real rows), N, K per stage (halves)
constexpr int STAGES = 4;
constexpr int A_BYTES = TM * TK * 2, B_BYTES = TN * TK * 2, STAGE_BYTES = A_BYTES + B_BYTES;
constexpr int CCH = TC_CCH;                       // epilogue chunk: 128 rows x 32 columns of C'
constexpr int C_BYTES = TM * CCH * 4;              // 16 KB per chunk buffer
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 2 * C_BYTES + 1024 + 256;
constexpr long long WAIT_CYCLES = 4000000000LL;  // ~2 s at 2 GHz

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait on an mbarrier phase; false (status bit 4, CTA abort flag raised) on timeout,
// and false at once when another role of the CTA has already given up
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int* status,
                                          volatile int* abort) {
  long long t0 = clock64();
  while (!mbar_test(bar, parity)) {
    if (*abort) return false;
    if (clock64() - t0 > WAIT_CYCLES) {
      atomicOr(status, 4);
      *abort = 1;
      return false;
    }
  }
  return true;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// C' += (chunk in shared memory), element-wise FP32 add performed by the TMA unit
__device__ __forceinline__ void tma_reduce_add_2d(const CUtensorMap* map, int x, int y, uint32_t src) {
  asm volatile(
      "cp.reduce.async.bulk.tensor.2d.global.shared::cta.add.tile.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
          (uint64_t)map),
      "r"(x), "r"(y), "r"(src)
      : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read1() { asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait0() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// shared-memory matrix descriptor: K-major operand, 128-byte swizzle, 8-row atoms of 1024 B
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFF) >> 4);   // start address
  d |= (uint64_t)1 << 16;                    // leading byte offset (unused for this layout)
  d |= (uint64_t)(1024 >> 4) << 32;          // stride byte offset: next 8-row atom
  d |= (uint64_t)1 << 46;                    // descriptor version
  d |= (uint64_t)2 << 61;                    // swizzle: 128 B
  return d;
}

// instruction descriptor: D f32, A/B f16, both K-major, M = 128, N = 256
__host__ __device__ constexpr uint32_t idesc_f16() {
  return (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(TN >> 3) << 17) | ((uint32_t)(TM >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                        uint32_t accum) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.u32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accum)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// C' (real view, ldc floats) -= A' B' over a grid of 128 x 256 tiles, persistent CTAs.
// Warp roles: warp 0 lane 0 issues TMA loads into a STAGES-deep ring, warp 1 lane 0 issues
// tcgen05.mma into one of two 256-column TMEM accumulators, warps 2..5 drain the other
// accumulator (tcgen05.ld -> C' -= D) so that the epilogue of tile t overlaps the loads and
// MMAs of tile t+1.  Barriers: full/empty per stage (TMA <-> MMA), tfull/tempty per
// accumulator (MMA <-> epilogue).  The update region, its tiles and their order: TcRegion,
// tc_tile_at (tc_tiles.h).
__global__ void __launch_bounds__(192, 1)
    k_tc_gemm(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
              const __grid_constant__ CUtensorMap tmC0, const __grid_constant__ CUtensorMap tmC1,
              const TcRegion Rg, const float* __restrict__ inv_sa, const float* __restrict__ inv_sb, int nk,
              int* status) {
  extern __shared__ unsigned char smraw[];
  const uint32_t base = (smem_u32(smraw) + 1023u) & ~1023u;
  unsigned char* gbase = smraw + (base - smem_u32(smraw));
  uint64_t* bars = reinterpret_cast<uint64_t*>(gbase + STAGES * STAGE_BYTES);
  // C' chunk buffers follow the operand ring; then the barriers:
  // full[STAGES], empty[STAGES], tfull[2], tempty[2], done
  const uint32_t cbuf0 = base + STAGES * STAGE_BYTES;
  float* cbuf_g = reinterpret_cast<float*>(gbase + STAGES * STAGE_BYTES);
  bars = reinterpret_cast<uint64_t*>(gbase + STAGES * STAGE_BYTES + 2 * C_BYTES);
  const int B_FULL = 0, B_EMPTY = STAGES, B_TFULL = 2 * STAGES, B_TEMPTY = 2 * STAGES + 2,
            B_DONE = 2 * STAGES + 4;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 7);
  __shared__ int s_abort_mem;
  volatile int* s_abort = &s_abort_mem;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntiles = Rg.ntiles;
  const int unit0 = (int)blockIdx.x;  // first tile of this CTA
  const int nunits = (int)gridDim.x;
  auto tile_at = [&](int tile, int& r, int& m0, int& n0) -> bool { return tc_tile_at(Rg, tile, r, m0, n0); };

  if (threadIdx.x == 0) {
    *s_abort = 0;
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(smem_u32(bars + B_FULL + s), 1);
      mbar_init(smem_u32(bars + B_EMPTY + s), 1);
    }
    for (int a = 0; a < 2; ++a) {
      mbar_init(smem_u32(bars + B_TFULL + a), 1);
      mbar_init(smem_u32(bars + B_TEMPTY + a), 4);  // one arrival per epilogue warp
    }
    mbar_init(smem_u32(bars + B_DONE), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(2 * TN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // ---- TMA producer
    uint32_t it = 0;
    for (int tile = unit0; tile < ntiles && !*s_abort; tile += nunits) {
      int rr, m0, n0;
      tile_at(tile, rr, m0, n0);
      for (int kb = 0; kb < nk; ++kb, ++it) {
        const int s = it % STAGES;
        const uint32_t ph = (it / STAGES) & 1;
        if (!mbar_wait(smem_u32(bars + B_EMPTY + s), ph ^ 1, status, s_abort)) break;
        const uint32_t sa = base + s * STAGE_BYTES, sb = sa + A_BYTES;
        const uint32_t full = smem_u32(bars + B_FULL + s);
        mbar_expect_tx(full, STAGE_BYTES);
        tma_load_2d(sa, &tmA, kb * TK, m0, full);
        tma_load_2d(sb, &tmB, kb * TK, Rg.b_col[rr] + n0, full);
      }
    }
    // no copy may still be landing in shared memory when the CTA exits: wait (bounded,
    // whatever the abort state) for the last load issued into each stage
    int no_abort = 0;
    for (uint32_t j = it > (uint32_t)STAGES ? it - STAGES : 0; j < it; ++j)
      mbar_wait(smem_u32(bars + B_FULL + j % STAGES), (j / STAGES) & 1, status, &no_abort);
  } else if (warp == 1 && lane == 0) {
    // ---- MMA issuer
    const uint32_t idesc = idesc_f16();
    uint32_t it = 0;
    int t = 0;
    for (int tile = unit0; tile < ntiles && !*s_abort; tile += nunits, ++t) {
      const int a = t & 1;
      const uint32_t aph = (t >> 1) & 1;
      if (!mbar_wait(smem_u32(bars + B_TEMPTY + a), aph ^ 1, status, s_abort)) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t acc = tmem + (uint32_t)(a * TN);
      for (int kb = 0; kb < nk; ++kb, ++it) {
        const int s = it % STAGES;
        const uint32_t ph = (it / STAGES) & 1;
        if (!mbar_wait(smem_u32(bars + B_FULL + s), ph, status, s_abort)) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t sa = base + s * STAGE_BYTES, sb = sa + A_BYTES;
#pragma unroll
        for (int kk = 0; kk < TK / 16; ++kk)
          mma_f16(acc, smem_desc(sa + kk * 32), smem_desc(sb + kk * 32), idesc, (kb | kk) ? 1u : 0u);
        mma_commit(smem_u32(bars + B_EMPTY + s));
      }
      if (*s_abort) break;
      mma_commit(smem_u32(bars + B_TFULL + a));
    }
    // every MMA issued above has completed once this barrier phase does (waited for even
    // after an abort, with its own budget, so that no MMA runs when TMEM is released)
    mma_commit(smem_u32(bars + B_DONE));
    int no_abort = 0;
    mbar_wait(smem_u32(bars + B_DONE), 0, status, &no_abort);
  } else if (warp >= 2) {
    // ---- epilogue: warp w owns TMEM lanes 32*(w%4) .. +31 (= tile rows).  Each 128 x 32
    // chunk of -D / (s t) goes through one of two shared-memory buffers (column-major like
    // C') and is added to C' by a TMA reduce-add: C' is never loaded into the SM.  A buffer
    // is rewritten once the reduce issued from it two chunks earlier has read it.
    const int q = warp & 3;
    const bool leader = (warp == 2 && lane == 0);
    // the chunk buffers alternate over this CTA's whole chunk sequence (tiles may end on an odd
    // chunk), so that the buffer being refilled is always the one of two reduces back
    int gc = 0;
    int t = 0;
    for (int tile = unit0; tile < ntiles; tile += nunits, ++t) {
      const int a = t & 1;
      const uint32_t aph = (t >> 1) & 1;
      int rr, m0, n0;
      const bool valid = tile_at(tile, rr, m0, n0);
      const CUtensorMap* tmC = rr ? &tmC1 : &tmC0;
      const int m_rows = Rg.m_rows[rr], n_cols = Rg.n_cols[rr];
      if (!mbar_wait(smem_u32(bars + B_TFULL + a), aph, status, s_abort)) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (!valid) {  // nothing to store: hand the accumulator straight back
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncwarp();
        if (lane == 0)
          asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bars + B_TEMPTY + a)) : "memory");
        continue;
      }
      const uint32_t tbase = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(a * TN);
      const int row = q * 32 + lane;
      // -1 / s of this thread's row (rows beyond the block are clipped by the TMA reduce)
      const float rs = m0 + row < m_rows ? -inv_sa[(m0 + row) >> 1] : 0.f;
      // chunks that hold a column of the rectangle (narrow updates leave the rest of the
      // accumulator unread: its reduce-adds would lie wholly outside the tensor map)
      const int nchv = tc_tile_chunks(n_cols, n0);
      for (int c = 0; c < nchv; ++c, ++gc) {
        const int b = gc & 1;
        float v[CCH];
        tmem_ld16(tbase + (uint32_t)(c * CCH), v);
        tmem_ld16(tbase + (uint32_t)(c * CCH + 16), v + 16);
        if (c == nchv - 1) {
          // accumulator read: hand it back to the MMA warp
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
          __syncwarp();
          if (lane == 0)
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bars + B_TEMPTY + a)) : "memory");
        }
        // 1 / t of the chunk's columns, one per lane, broadcast by shuffles
        const int gcol = n0 + c * CCH + lane;
        const float cs = gcol < n_cols ? inv_sb[Rg.b_col[rr] + gcol] : 0.f;
        if (leader) bulk_wait_read1();  // the reduce two chunks back has read buffer b
        asm volatile("bar.sync 1, 128;" ::: "memory");
        float* cb = cbuf_g + b * (TM * CCH);
#pragma unroll
        for (int i = 0; i < CCH; ++i) cb[i * TM + row] = v[i] * __shfl_sync(0xffffffffu, cs, i) * rs;
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("bar.sync 1, 128;" ::: "memory");
        if (leader) {
          tma_reduce_add_2d(tmC, Rg.c_row0 + m0, Rg.c_col0[rr] + n0 + c * CCH, cbuf0 + b * C_BYTES);
          bulk_commit();
        }
      }
    }
    if (leader) bulk_wait0();
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * TN) : "memory");
  }
}

// A' (K-major; rows 2m, 2m+1 hold 2K halves): [[ar, -ai], [ai, ar]] blocks times s_m;
// inv_sa[m] = 1 / s_m.  A CTA takes 32 rows: the row maxima first, then 64-column slices
// transposed through shared memory so that every warp writes whole row segments.
__device__ __forceinline__ void expand_h(int bid, const float2* A, int64_t lda, int M, int K, __half2* Ap,
                                         float* inv_sa) {
  __shared__ float red[8][33];
  __shared__ float2 tile[32][65];
  __shared__ float s_scale[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int m0 = bid * 32, m = m0 + lane;
  float mx = 0.f;
  if (m < M)
    for (int k = w; k < K; k += 8) {
      const float2 a = A[m + (int64_t)k * lda];
      mx = fmaxf(mx, fmaxf(fabsf(a.x), fabsf(a.y)));
    }
  red[w][lane] = mx;
  __syncthreads();
  if (w == 0) {
    for (int j = 1; j < 8; ++j) mx = fmaxf(mx, red[j][lane]);
    const int sh = tc_scale_shift(mx);
    s_scale[lane] = ldexpf(1.f, sh);
    if (m < M) inv_sa[m] = ldexpf(1.f, -sh);
  }
  __syncthreads();
  for (int k0 = 0; k0 < K; k0 += 64) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int k = k0 + w + 8 * j;
      tile[lane][w + 8 * j] = (m < M && k < K) ? A[m + (int64_t)k * lda] : make_float2(0.f, 0.f);
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int r = w + 8 * i, mr = m0 + r;
      if (mr < M) {
        const float sc = s_scale[r];
        __half2* row0 = Ap + (int64_t)(2 * mr) * K;  // 2K halves = K half2 per row
        __half2* row1 = row0 + K;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int kk = lane + 32 * h, k = k0 + kk;
          if (k < K) {
            const float2 a = tile[r][kk];
            row0[k] = __floats2half2_rn(a.x * sc, -a.y * sc);
            row1[k] = __floats2half2_rn(a.y * sc, a.x * sc);
          }
        }
      }
    }
    __syncthreads();
  }
}

// B' (column j: 2K halves, (re, im) per k) times t_j; inv_sb[j] = 1 / t_j.  One warp per column.
__device__ __forceinline__ void convert_bh(int bid, const float2* B, int64_t lda, int K, int N, __half2* Bp,
                                           float* inv_sb) {
  const int lane = threadIdx.x & 31;
  const int j = bid * 8 + (threadIdx.x >> 5);
  if (j >= N) return;
  const float2* col = B + (int64_t)j * lda;
  float mx = 0.f;
  for (int k = lane; k < K; k += 32) {
    const float2 a = col[k];
    mx = fmaxf(mx, fmaxf(fabsf(a.x), fabsf(a.y)));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  const int sh = tc_scale_shift(mx);
  const float sc = ldexpf(1.f, sh);
  if (lane == 0) inv_sb[j] = ldexpf(1.f, -sh);
  __half2* out = Bp + (int64_t)j * K;
  for (int k = lane; k < K; k += 32) {
    const float2 a = col[k];
    out[k] = __floats2half2_rn(a.x * sc, a.y * sc);
  }
}

// Both FP16 operands of a symmetric update C[r0.., r0..] -= L D L^T from the same rows of L
// (M x K at L, ld lda; B' takes the first N <= M of them), D the pivots dg[k (lda + 1)]:
//   A' rows 2m, 2m+1 = [[re, -im], [im, re]] of L[m][k] times s_m (as expand_h),
//   B' column m = d_k L[m][k] times t_m (m < N);
// s_m, t_m put the largest |re|, |im| of the row of L resp. D-scaled row into [2^13, 2^14).
// A CTA takes 32 rows: one pass for both maxima, one pass through 32 x 64 shared-memory tiles
// (coalesced along the rows of L) writing both operands; the pivots are staged once.
__global__ void __launch_bounds__(256) k_prep_sym(const float2* L, const float2* dg, int64_t lda, int M, int N, int K,
                                                  __half2* Ap, float* inv_sa, __half2* Bp, float* inv_sb) {
  __shared__ float red[2][8][33];
  __shared__ float2 tile[32][65];
  __shared__ float s_sa[32], s_sb[32];
  __shared__ float2 s_d[TC_SYM_KMAX];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int m0 = blockIdx.x * 32, m = m0 + lane;
  for (int k = threadIdx.x; k < K; k += 256) s_d[k] = dg[(int64_t)k * (lda + 1)];
  __syncthreads();
  float ma = 0.f, mb = 0.f;
  if (m < M)
    for (int k = w; k < K; k += 8) {
      const float2 a = L[m + (int64_t)k * lda], d = s_d[k];
      const float re = a.x * d.x - a.y * d.y, im = a.x * d.y + a.y * d.x;
      ma = fmaxf(ma, fmaxf(fabsf(a.x), fabsf(a.y)));
      mb = fmaxf(mb, fmaxf(fabsf(re), fabsf(im)));
    }
  red[0][w][lane] = ma;
  red[1][w][lane] = mb;
  __syncthreads();
  if (w == 0) {
    for (int q = 1; q < 8; ++q) {
      ma = fmaxf(ma, red[0][q][lane]);
      mb = fmaxf(mb, red[1][q][lane]);
    }
    const int sha = tc_scale_shift(ma), shb = tc_scale_shift(mb);
    s_sa[lane] = ldexpf(1.f, sha);
    s_sb[lane] = ldexpf(1.f, shb);
    if (m < M) inv_sa[m] = ldexpf(1.f, -sha);
    if (m < N) inv_sb[m] = ldexpf(1.f, -shb);
  }
  __syncthreads();
  for (int k0 = 0; k0 < K; k0 += 64) {
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int k = k0 + w + 8 * q;
      tile[lane][w + 8 * q] = (m < M && k < K) ? L[m + (int64_t)k * lda] : make_float2(0.f, 0.f);
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int r = w + 8 * i, mr = m0 + r;
      if (mr < M) {
        const float sa = s_sa[r], sb = s_sb[r];
        __half2* row0 = Ap + (int64_t)(2 * mr) * K;
        __half2* row1 = row0 + K;
        __half2* col = Bp + (int64_t)mr * K;
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
          const int kk = lane + 32 * hh, k = k0 + kk;
          if (k < K) {
            const float2 a = tile[r][kk];
            row0[k] = __floats2half2_rn(a.x * sa, -a.y * sa);
            row1[k] = __floats2half2_rn(a.y * sa, a.x * sa);
            if (mr < N) {
              const float2 d = s_d[k];
              col[k] = __floats2half2_rn((a.x * d.x - a.y * d.y) * sb, (a.x * d.y + a.y * d.x) * sb);
            }
          }
        }
      }
    }
    __syncthreads();
  }
}

// both operands in one launch: CTAs [0, nA) expand 32 rows of A each, the rest convert 8
// columns of B each
__global__ void __launch_bounds__(256) k_prep_h(const float2* A, const float2* B, int64_t lda, int M, int N, int K,
                                                __half2* Ap, float* inv_sa, __half2* Bp, float* inv_sb, int nA) {
  if ((int)blockIdx.x < nA)
    expand_h(blockIdx.x, A, lda, M, K, Ap, inv_sa);
  else
    convert_bh(blockIdx.x - nA, B, lda, K, N, Bp, inv_sb);
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// looked up once per process; std::call_once makes concurrent first calls (several host
// threads, one per serving slot) see the finished result
EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

bool make_map(CUtensorMap* m, const void* base, uint64_t dim0, uint64_t dim1, uint64_t stride1_bytes,
              uint32_t box0, uint32_t box1, bool swizzle, CUtensorMapDataType dt) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[2] = {dim0, dim1};
  cuuint64_t strides[1] = {stride1_bytes};
  cuuint32_t box[2] = {box0, box1};
  cuuint32_t es[2] = {1, 1};
  CUresult r = fn(m, dt, 2, const_cast<void*>(base), dims, strides, box, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE,
                  swizzle ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

}  // namespace

// is the tensor-core path usable for this update (alignment rules of TMA)?
bool tc_gemm_supported(const void* A, int64_t lda, int K) {
  if (!encode_fn()) return false;
  if ((reinterpret_cast<uintptr_t>(A) & 15) != 0) return false;
  if (lda % 2 != 0) return false;  // column stride of the real view: multiple of 16 B
  if (K % 32 != 0) return false;   // 2K halves = whole 64-half K stages
  return true;
}

// bytes of workspace tc_gemm_sub needs for an M x K by K x N update
size_t tc_gemm_work_bytes(int64_t M, int64_t N, int K) {
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  return al((size_t)M * K * 8) + al((size_t)N * K * 4) + al((size_t)M * 4) + al((size_t)N * 4);
}

void tc_gemm_operands(void* work, int64_t M, int64_t N, int K, void** Ap, float** inv_sa, void** Bp,
                      float** inv_sb) {
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  char* w = static_cast<char*>(work);
  *Ap = w;
  *Bp = w + al((size_t)M * K * 8);
  *inv_sa = reinterpret_cast<float*>(w + al((size_t)M * K * 8) + al((size_t)N * K * 4));
  *inv_sb = reinterpret_cast<float*>(reinterpret_cast<char*>(*inv_sa) + al((size_t)M * 4));
}

// One tensor-core update of the matrix Mat (ld lda), C -= A B over one or two rectangles of C
// sharing the operands (see TcRegion), A = Mat[rowA.., colA..] (M0 x K).
//   LU:        B = Mat[colA.., colB..] (K x (N0 + N1))
//   symmetric: B = D L^T with L = Mat[rowB.., colA..] (N0 x K) and D the pivots
//              Mat[colA + k, colA + k]; C columns from colB = rowB; lower: only the tiles on or
//              below the diagonal (rowA = rowB, M0 = N0, one rectangle)
// prepped: the FP16 operands are already in work (tc_gemm_operands layout, written by the
// kernel that produced A and B).
// a_skip (prepped only): the operands were written for a_skip + M0 rows of A and the update
// uses the last M0 of them
struct TcUpdate {
  int64_t rowA, colA, colB, M0, N0, M1, N1;
  int K;
  bool sym, lower, prepped;
  int64_t a_skip = 0;
};

static int tc_gemm_run(beast_ctx* ctx, float2* Mat, int64_t lda, const TcUpdate& u, void* work, size_t work_bytes) {
  cudaStream_t st = ctx->stream;
  const int64_t rowA = u.rowA, colA = u.colA, colB = u.colB, M0 = u.M0, N0 = u.N0, M1 = u.M1, N1 = u.N1;
  const int K = u.K;
  const int64_t N = N0 + N1;
  // TMA: the first C' row (2 rowA floats) must start on 16 bytes
  if ((2 * rowA) % 4 != 0 || K % 32 != 0 || M1 > M0 || 2 * (rowA + M0) > INT32_MAX || colB + N > INT32_MAX)
    return beast_fail(ctx, BEAST_ERR_ARG, "tensor-core update: unaligned block");
  if (u.lower && (u.sym == false || rowA != colB || M0 != N0 || N1 != 0))
    return beast_fail(ctx, BEAST_ERR_ARG, "tensor-core update: lower-triangle tiles need a diagonal square");
  if (u.a_skip < 0 || (u.a_skip > 0 && !u.prepped) || tc_gemm_work_bytes(M0 + u.a_skip, N, K) > work_bytes)
    return beast_fail(ctx, BEAST_ERR_ARG, "tensor-core update: workspace too small");
  {
    // the kernel's shared-memory attribute, set once per device (serving slots may make their
    // first factorisation concurrently from several host threads)
    static std::mutex mtx;
    static bool attr_done[64] = {false};
    const int dev = ctx->device;
    if (dev < 0 || dev >= 64) return beast_fail(ctx, BEAST_ERR_ARG, "tensor-core update: device index out of range");
    std::lock_guard<std::mutex> lk(mtx);
    if (!attr_done[dev]) {
      BEAST_CUDA_TRY(ctx, cudaFuncSetAttribute(k_tc_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
      attr_done[dev] = true;
    }
  }
  void *Apv, *Bpv;
  float *inv_sa, *inv_sb;
  tc_gemm_operands(work, M0 + u.a_skip, N, K, &Apv, &inv_sa, &Bpv, &inv_sb);
  __half2* Ap = static_cast<__half2*>(Apv) + 2 * u.a_skip * K;  // A' rows 2m, 2m+1 of K half2 each
  __half2* Bp = static_cast<__half2*>(Bpv);
  inv_sa += u.a_skip;
  if (!u.prepped) {
    // FP16 operands: A read and A' written (2 x 4 B per complex element), B read and B' written
    ProfScope ps(ctx, PK_CONVERT, (double)M0 * K * 16.0 + (double)N * K * 12.0);
    const int nA = (int)((M0 + 31) / 32);
    if (u.sym) {
      if (colB != rowA || N > M0 || K > TC_SYM_KMAX)
        return beast_fail(ctx, BEAST_ERR_ARG, "symmetric update: operands must come from the same rows");
      k_prep_sym<<<(unsigned)nA, 256, 0, st>>>(Mat + rowA + colA * lda, Mat + colA + colA * lda, lda, (int)M0,
                                               (int)N, K, Ap, inv_sa, Bp, inv_sb);
    } else {
      const int nB = (int)((N + 7) / 8);
      k_prep_h<<<(unsigned)(nA + nB), 256, 0, st>>>(Mat + rowA + colA * lda, Mat + colA + colB * lda, lda,
                                                    (int)M0, (int)N, K, Ap, inv_sa, Bp, inv_sb, nA);
    }
    BEAST_CUDA_TRY(ctx, cudaGetLastError());
  }
  CUtensorMap tmA, tmB, tmC0, tmC1;
  // A': 2K halves per row (x), 2 M0 rows (y); B': 2K halves per column (x), N columns (y)
  if (!make_map(&tmA, Ap, (uint64_t)2 * K, (uint64_t)2 * M0, (uint64_t)2 * K * 2, TK, TM, true,
                CU_TENSOR_MAP_DATA_TYPE_FLOAT16))
    return beast_fail(ctx, BEAST_ERR_CUDA, "tensor map encode (A') failed");
  if (!make_map(&tmB, Bp, (uint64_t)2 * K, (uint64_t)N, (uint64_t)2 * K * 2, TK, TN, true,
                CU_TENSOR_MAP_DATA_TYPE_FLOAT16))
    return beast_fail(ctx, BEAST_ERR_CUDA, "tensor map encode (B') failed");
  // C': real view clipped to each rectangle (rows up to 2(rowA + M_r), columns up to its last
  // column): the reduce-adds never touch anything outside the rectangle
  const float* real = reinterpret_cast<const float*>(Mat);
  if (!make_map(&tmC0, real, (uint64_t)2 * (rowA + M0), (uint64_t)(colB + N0), (uint64_t)2 * lda * 4, TM, CCH,
                false, CU_TENSOR_MAP_DATA_TYPE_FLOAT32))
    return beast_fail(ctx, BEAST_ERR_CUDA, "tensor map encode (C') failed");
  tmC1 = tmC0;
  if (N1 > 0 && M1 > 0 &&
      !make_map(&tmC1, real, (uint64_t)2 * (rowA + M1), (uint64_t)(colB + N), (uint64_t)2 * lda * 4, TM, CCH, false,
                CU_TENSOR_MAP_DATA_TYPE_FLOAT32))
    return beast_fail(ctx, BEAST_ERR_CUDA, "tensor map encode (C') failed");
  TcRegion Rg;
  Rg.lower = u.lower ? 1 : 0;
  Rg.c_row0 = (int)(2 * rowA);
  Rg.m_rows[0] = (int)(2 * M0);
  Rg.n_cols[0] = (int)N0;
  Rg.b_col[0] = 0;
  Rg.c_col0[0] = (int)colB;
  Rg.m_rows[1] = (int)(2 * M1);
  Rg.n_cols[1] = (int)N1;
  Rg.b_col[1] = (int)N0;
  Rg.c_col0[1] = (int)(colB + N0);
  tc_region_count(Rg);
  if (Rg.ntiles == 0) return BEAST_OK;
  const int nk = (2 * K) / TK;
  // algorithmic work: 8 K per complex element of the region (the lower triangle: half the square)
  ProfScope ps(ctx, PK_TCGEMM,
               8.0 * K * (u.lower ? 0.5 * (double)M0 * N0 : (double)M0 * N0 + (double)M1 * N1));
  const int grid = std::min(Rg.ntiles, std::max(1, ctx->num_sms - ctx->tc_sm_reserve));
  k_tc_gemm<<<grid, 192, SMEM_BYTES, st>>>(tmA, tmB, tmC0, tmC1, Rg, inv_sa, inv_sb, nk, ctx->d_flag);
  BEAST_CUDA_TRY(ctx, cudaGetLastError());
  return BEAST_OK;
}

// C -= A B (complex64) for the LU updates, over an L-shaped region of C:
//   A at (rowA, colA) of the matrix, M0 x K;  B at (colA, colB), K x (N0 + N1);
//   rectangle 0: C[rowA : rowA+M0, colB : colB+N0]     = A[0:M0]  B[:, 0:N0]
//   rectangle 1: C[rowA : rowA+M1, colB+N0 : +N1]      = A[0:M1]  B[:, N0:N0+N1]   (M1 <= M0)
// (N1 = 0: one rectangle).  work: tc_gemm_work_bytes(M0, N0 + N1, K) bytes or more.
int tc_gemm_sub(beast_ctx* ctx, float2* Mat, int64_t lda, int64_t rowA, int64_t colA, int64_t colB,
                int64_t M0, int64_t N0, int64_t M1, int64_t N1, int K, void* work, size_t work_bytes,
                bool prepped) {
  TcUpdate u{rowA, colA, colB, M0, N0, M1, N1, K, false, false, prepped};
  return tc_gemm_run(ctx, Mat, lda, u, work, work_bytes);
}

// Symmetric update of an LDL^T-type factorisation: C[rowA.., rowB..] (M0 x N0) -= L1 D L2^T
// with L1 = Mat[rowA.., colA..] (M0 x K), L2 = Mat[rowB.., colA..] (N0 x K), D the pivots on
// the diagonal of Mat at colA..; lower: only the tiles on or below the diagonal (rowA = rowB,
// M0 = N0).
int tc_gemm_sym(beast_ctx* ctx, float2* Mat, int64_t lda, int64_t rowA, int64_t colA, int64_t rowB, int64_t M0,
                int64_t N0, int K, bool lower, void* work, size_t work_bytes, bool prepped, int64_t a_skip) {
  TcUpdate u{rowA, colA, rowB, M0, N0, 0, 0, K, true, lower, prepped, a_skip};
  return tc_gemm_run(ctx, Mat, lda, u, work, work_bytes);
}
