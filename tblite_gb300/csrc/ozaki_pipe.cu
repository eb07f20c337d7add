// Pipelined FP64-accurate split GEMM on the BF16 tensor cores for the one-molecule path.
//
// Same splitting as ozaki.cu: eight 7-bit slices per FP64 value, x = 2^e sum_p a_p 2^-7p, stored
// pre-scaled in BF16, and the 36 exact slice products a_p b_q with p + q <= 7 (zero based).  The
// operands are split once per matrix instead of once per tile pair, and the products are grouped
// so that each tensor-core instruction is wide:
//
//   psplit   turns a matrix into a slice image: per line (row of op(A) or column of op(B)) a
//            power-of-two exponent, and the eight BF16 slices laid out exactly as the tensor
//            cores read them from shared memory, K-major lines of 64 bytes with the 64-byte
//            swizzle: image[k chunk of 32][slice][line block of 64][64 x 64 bytes];
//   pgemm    (kernel k_opipe) one 128 x 64 output tile per CTA, 10 warps.  Warp 0 streams the
//            slices of each k chunk (96 KB: A 64 KB, B 32 KB) with cp.async.bulk into a
//            two-stage shared-memory ring (mbarrier complete_tx).  Warp 1 issues the MMAs: the B
//            slices of a stage lie one after another, so a_p times [b_q0 .. b_q0+3] is a single
//            M 128 x N 256 x K 16 tcgen05.mma whose four 64-column blocks land in the TMEM
//            accumulators of the levels p + q0 .. p + q0 + 3 (one accumulator of 64 columns per
//            level 0..7, 512 columns); 13 MMAs per k step instead of 36.  Warps 2..9 drain the
//            levels 0..5 every 5 chunks (160 values of k): they hold exact integers (at most 6
//            products of < 2^14 each per k: < 2^24) that go into one int64 per element.  The
//            levels 6..7 (< 2^-42 of the leading level) stay in FP32 over the whole of k (their
//            rounding is < 2^-56 of the result) and are read with the output at the end.
//
// Every wait is bounded; a wait that runs out sets a CTA-wide abort flag, the other roles leave
// their loops, copies and MMAs still in flight are waited for (bounded), TMEM is freed and the
// status word is set.  Tiles are visited in groups of 8 row blocks so that the slices a wave of
// CTAs reads stay in L2.  Symmetric products compute the tiles on and below the diagonal and
// write each element also to its mirror position.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <stdexcept>
#include <string>

#include "engine.h"

namespace tb {

namespace {

constexpr int PP_M = 128, PP_N = 64, PP_KC = 32, PP_FLUSH = 5, PP_THREADS = 320;
constexpr int PP_LEVELS = 8;    // TMEM accumulators, one per level p + q = 0..7
constexpr int PP_EXACT = 6;     // levels 0..5 are drained as exact integers
constexpr int PP_KMAX = 12288;  // |int64 level sums| < 1.02 * 2^49 K < 2^63
constexpr int PP_STAGES = 2;    // the producer's bookkeeping below assumes two
constexpr int PP_A_BYTES = 8 * 8192;  // 8 slices x 128 lines x 64 B
constexpr int PP_B_BYTES = 8 * 4096;  // 8 slices x 64 lines x 64 B
constexpr int PP_STAGE_BYTES = PP_A_BYTES + PP_B_BYTES;
constexpr int PP_SMEM = PP_STAGES * PP_STAGE_BYTES + 1024;
constexpr int PP_TMEM_COLS = 512;
static_assert(PP_LEVELS * PP_N == PP_TMEM_COLS, "one 64-column accumulator per level");
constexpr int PP_GROUP = 8;  // row blocks per tile group
constexpr int PP_WAIT = 1 << 22;
// polls of a pipeline wait (stage full / empty, accumulators ready / free) before it gives up
// and aborts the tile; the drains of copies and MMAs in flight after an abort always use
// PP_WAIT.  Settable for tests (tblite_gb300_set_pipeline_wait_limit) so that a wait runs out
// and the abort path, the status word and the hand-off can be checked.
__device__ int g_pipe_wait_limit = PP_WAIT;
// FP64-equivalent flop (2 m n K per output tile that ran) of the batched squarings since load
__device__ unsigned long long g_pipe_batch_flops = 0;

void ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess)
    throw std::runtime_error(std::string("CUDA error '") + cudaGetErrorString(e) + "' in " + what);
}

__device__ __forceinline__ uint32_t su32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
// shared-memory matrix descriptor (K-major, descriptor version 1): lines of 64 bytes (32 BF16 of
// k), 8-line atoms 512 B apart, the 16-byte chunks of line r permuted by chunk ^ ((r >> 1) & 3)
// (the 64-byte swizzle); a k step of 16 moves the start by 32 bytes
__device__ __forceinline__ uint64_t sdesc_sw64(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)1 << 16) | ((uint64_t)(512 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)4 << 61);
}
__device__ __forceinline__ bool try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait; gives up early once another role has aborted (abort != nullptr)
__device__ __forceinline__ bool wait_bar(uint32_t bar, uint32_t parity, volatile int* abort) {
  const int limit = abort ? g_pipe_wait_limit : PP_WAIT;
  for (int it = 0; it < limit; ++it) {
    if (try_wait(bar, parity)) return true;
    if (abort && *abort) return false;
  }
  return false;
}

// 16 consecutive TMEM columns of this thread's lane (one row of the tile) into v
__device__ __forceinline__ void tmem_ld16(uint32_t addr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15])
      : "r"(addr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// |x| 2^(56 - e) as an integer (< 2^56 for |x| < 2^e): zero and subnormals give zero
__device__ __forceinline__ uint64_t fixed_bits(uint64_t bits, int e) {
  const int ex = (int)((bits >> 52) & 0x7FF);
  if (ex == 0) return 0ull;
  const uint64_t m = (bits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  const int sh = ex - e - 1019;
  return sh >= 0 ? m << sh : (sh > -64 ? m >> (-sh) : 0ull);
}

// a - b of two packed BF16 pairs (the bits of both), one BF16x2 instruction
__device__ __forceinline__ uint32_t bf16x2_sub(uint32_t a, uint32_t b) {
  union {
    uint32_t u;
    __nv_bfloat162 v;
  } x, y, r;
  x.u = a;
  y.u = b;
  r.v = __hsub2(x.v, y.v);
  return r.u;
}

// |x| as bits: for non-negative doubles the unsigned order of the bit patterns is the numeric
// order, so line maxima are integer maxima (no FP64 instruction, which this GPU issues at 1/64
// of the FP32 rate); e = ilogb(max) + 1 is the biased exponent field minus 1022 for a normal
// maximum
__device__ __forceinline__ unsigned long long abs_bits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
}
__device__ __forceinline__ int exp_of_max(unsigned long long mb) {
  const int mexp = (int)(mb >> 52);
  return mb == 0ull ? 0 : mexp > 0 ? mexp - 1022 : ilogb(__longlong_as_double((long long)mb)) + 1;
}

// ---- exponents: e = ilogb(max |x|) + 1 of every line ------------------------------------------
// lines contiguous in memory (element (i, k) at M[i + k ld]): 32 lines per block, the 8 warps
// take every 8th k (coalesced 256-byte rows), then a shared-memory reduction
__device__ __forceinline__ void pexp_rows_dev(const double* __restrict__ M, int ld, int lines,
                                              int K, int Lp, int* e, int blk) {
  __shared__ unsigned long long part[8][33];
  const int li = threadIdx.x & 31, kg = threadIdx.x >> 5;
  const int i = blk * 32 + li;
  unsigned long long mx = 0ull;
  if (i < lines)
    for (int k = kg; k < K; k += 8) mx = max(mx, abs_bits(M[i + (size_t)k * ld]));
  part[kg][li] = mx;
  __syncthreads();
  if (kg == 0 && i < Lp) {
    for (int g = 1; g < 8; ++g) mx = max(mx, part[g][li]);
    e[i] = exp_of_max(mx);
  }
}
__global__ void __launch_bounds__(256) k_pexp_rows(const double* __restrict__ M, int ld,
                                                   int lines, int K, int Lp, int* e) {
  pexp_rows_dev(M, ld, lines, K, Lp, e, blockIdx.x);
}
// k contiguous (element (i, k) at M[k + i ld]): one warp per line
__global__ void k_pexp_cols(const double* __restrict__ M, int ld, int lines, int K, int Lp,
                            int* e) {
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (i >= Lp) return;
  unsigned long long mx = 0ull;
  if (i < lines)
    for (int k = lane; k < K; k += 32) mx = max(mx, abs_bits(M[k + (size_t)i * ld]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0) e[i] = exp_of_max(mx);
}

// ---- slice image: one block per (64 lines, 32 k); the FP64 tile goes through shared memory so
// both memory orders read coalesced; each thread splits 8 consecutive k of one line
__device__ __forceinline__ void psplit_dev(const double* __restrict__ M, int ld, int kcontig,
                                           int lines, int K, int nlb, const int* __restrict__ e,
                                           uint16_t* img, int lb, int kc) {
  __shared__ double tile[64][33];
  const int t = threadIdx.x;
  const int l0 = lb * 64, k0 = kc * PP_KC;
  if (!kcontig) {
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int li = t & 63, kk = (t >> 6) + 4 * r;
      const int i = l0 + li, k = k0 + kk;
      tile[li][kk] = (i < lines && k < K) ? M[i + (size_t)k * ld] : 0.0;
    }
  } else {
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int kk = t & 31, li = (t >> 5) + 8 * r;
      const int i = l0 + li, k = k0 + kk;
      tile[li][kk] = (i < lines && k < K) ? M[k + (size_t)i * ld] : 0.0;
    }
  }
  __syncthreads();
  const int li = t & 63, g = t >> 6;  // k group of 8: 0..3
  const int i = l0 + li;
  const int ei = e[i];
  uint32_t w[8][4];
#pragma unroll
  for (int c = 0; c < 8; c += 2) {  // two neighbouring k per step, as in kb_sp2_slice
    uint32_t hh[2], ll[2], signs = 0u;
#pragma unroll
    for (int d = 0; d < 2; ++d) {
      const uint64_t bits = (uint64_t)__double_as_longlong(tile[li][8 * g + c + d]);
      signs |= (uint32_t)(bits >> 63) << (15 + 16 * d);
      const uint64_t Y = fixed_bits(bits, ei);  // |x| 2^(56 - e) < 2^56; zero and subnormals: 0
      hh[d] = (uint32_t)(Y >> 28);
      ll[d] = (uint32_t)Y & 0xFFFFFFFu;
    }
    const uint32_t R[4] = {__byte_perm(hh[0] >> 14, hh[1] >> 14, 0x5410),
                           __byte_perm(hh[0], hh[1], 0x5410),
                           __byte_perm(ll[0] >> 14, ll[1] >> 14, 0x5410),
                           __byte_perm(ll[0], ll[1], 0x5410)};
#pragma unroll
    for (int p = 0; p < 8; ++p) {
      const uint32_t bias = ((uint32_t)(134 - 7 * p) << 7) * 0x10001u;
      const uint32_t mag = ((R[p >> 1] >> ((p & 1) ? 0 : 7)) & 0x007F007Fu) | bias;
      w[p][c >> 1] = bf16x2_sub(mag, bias) | signs;
    }
  }
  // [k chunk][slice][line block][64 lines x 64 B, 16-byte chunks swizzled]
#pragma unroll
  for (int p = 0; p < 8; ++p) {
    const size_t off = (((size_t)kc * 8 + p) * nlb + lb) * 2048 + li * 32 +
                       ((g ^ ((li >> 1) & 3)) << 3);
    *reinterpret_cast<uint4*>(img + off) = make_uint4(w[p][0], w[p][1], w[p][2], w[p][3]);
  }
}
__global__ void __launch_bounds__(256) k_psplit(const double* __restrict__ M, int ld, int kcontig,
                                                int lines, int K, int nlb,
                                                const int* __restrict__ e, uint16_t* img) {
  psplit_dev(M, ld, kcontig, lines, K, nlb, e, img, blockIdx.x, blockIdx.y);
}

struct PipeArgs {
  const uint16_t* A;  // slice image of op(A) (lines = rows, nlbA line blocks of 64)
  const uint16_t* B;  // slice image of op(B) (lines = columns)
  const int* eA;
  const int* eB;
  int eshiftA;  // added to every exponent of A (scaling A by a power of two)
  int nlbA, nlbB;
  int M, N, nkc;  // nkc: k chunks of 32
  double* C;
  int ldc;
  int sym;
  int* status;
  // the projection iterate (opipe_tile<true>): C holds signed 64-bit fixed-point values in units
  // of 2^-SP2_FRAC instead of doubles (|D_ij| <= 1); sub2: C <- 2 C - product (the old element
  // read first), which turns D^2 into 2D - D^2 in place
  int sub2;
  int fixed;
};

// line exponent of every projection iterate: the spectrum of D stays in [0, 1], so every element
// has |x| <= 1 < 2^SP2_E and the slices hold x to an absolute 2^-55 (an FP64 iterate's own
// rounding is 2^-53 relative to its O(1) diagonal); an element at or above 2^SP2_E stops the
// molecule.  During the projection the iterate lives in Y as signed 64-bit integers W = x 2^55
// (SP2_FRAC fractional bits): |W| < 2^56, and the magnitude's two 28-bit halves are the slices'
// source directly.
constexpr int SP2_E = 1;
constexpr int SP2_FRAC = 56 - SP2_E;
constexpr long long SP2_BAD = (long long)0x8000000000000000ull;  // an element out of range

__device__ __forceinline__ int slice_off(int line, int k, int nlb) {
  // image[k chunk][slice][line block][64 lines x 32 k], 16-byte groups swizzled (slice 0)
  const int li = line & 63, g = (k >> 3) & 3;
  return (((k >> 5) * 8) * nlb + (line >> 6)) * 2048 + li * 32 + ((g ^ ((li >> 1) & 3)) << 3) +
         (k & 7);
}


// C element (i, j) of a finished tile from the exact levels T, the FP32 levels v6 + v7 and the
// scale 2^sc: C = (T + F 2^35) 2^(sc - 35), F = levels 6 + 7 summed in FP32 (F < 2^-42 of the
// result, so its rounding is below 2^-66); the power of two goes into the exponent field by an
// integer add where the result stays normal: three FP64 operations per element (two conversions
// and an add) instead of six
__device__ __forceinline__ double tile_value(long long T, uint32_t v6, uint32_t v7, int sc) {
  const float ff = (__uint_as_float(v6) + __uint_as_float(v7)) * 0x1p35f;
  const double sum = (double)T + (double)ff;
  const long long sb = __double_as_longlong(sum);
  const int se = (int)((sb >> 52) & 0x7FF);
  if (sum == 0.0) return 0.0;
  if (se > 0 && se + (sc - 35) > 0 && se + (sc - 35) < 2047)
    return __longlong_as_double(sb + ((long long)(sc - 35) << 52));
  return ldexp(sum, sc - 35);  // subnormal or out-of-range result: the general path
}

// one 128 x 64 output tile (number b in the grouped order) of the product a (FIXED: the
// projection's fixed-point epilogue, a.fixed set)
template <bool FIXED = false>
__device__ __forceinline__ void opipe_tile(const PipeArgs& a, int b) {
  // ---- tile of this CTA: groups of PP_GROUP row blocks, column blocks inside a group
  const int mt = (a.M + PP_M - 1) / PP_M, nt = (a.N + PP_N - 1) / PP_N;
  const int gid = b / (PP_GROUP * nt);
  const int first = gid * PP_GROUP;
  const int gsize = min(mt - first, PP_GROUP);
  const int inner = b - gid * PP_GROUP * nt;
  const int tm = first + inner % gsize, tn = inner / gsize;
  const int i0 = tm * PP_M, j0 = tn * PP_N;
  if (a.sym && i0 + PP_M - 1 < j0) return;  // strictly above the diagonal: mirrored

  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem =
      smem_raw + ((1024 - (su32(smem_raw) & 1023)) & 1023);  // 1 KB aligned stages
  __shared__ __align__(8) uint64_t full[PP_STAGES], empty[PP_STAGES], accf, accfree, fin;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  volatile int* abort = &abort_flag;

  if (tid == 0) {
    for (int s = 0; s < PP_STAGES; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&full[s])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&empty[s])));
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&accf)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 256;" ::"r"(su32(&accfree)));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&fin)));
    asm volatile("fence.mbarrier_init.release.cluster;");
    abort_flag = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 ::"r"(su32(&tmem_base)), "r"(PP_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_base;
  const int nkc = a.nkc;
  const int nwin = (nkc + PP_FLUSH - 1) / PP_FLUSH;

  if (warp == 0) {
    // ---- producer: one elected lane streams the slices of every k chunk
    if (lane == 0) {
      const int lbA = i0 / 64, lbB = j0 / 64;
      int last0 = -1, last1 = -1;  // last chunk issued into stage 0 / 1
      for (int c = 0; c < nkc; ++c) {
        const int s = c % PP_STAGES;
        if (c >= PP_STAGES &&
            !wait_bar(su32(&empty[s]), (uint32_t)(((c - PP_STAGES) / PP_STAGES) & 1), abort)) {
          if (!*abort) atomicExch(&abort_flag, 1);
          break;
        }
        const uint32_t bar = su32(&full[s]);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
                     "r"(PP_STAGE_BYTES)
                     : "memory");
        unsigned char* st = smem + (size_t)s * PP_STAGE_BYTES;
        {  // per slice: A 8 KB (two line blocks), B 4 KB
#pragma unroll 1
          for (int p = 0; p < 8; ++p) {
            const size_t blk = (size_t)c * 8 + p;
            const uint16_t* srcA = a.A + (blk * a.nlbA + lbA) * 2048;
            const uint16_t* srcB = a.B + (blk * a.nlbB + lbB) * 2048;
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], "
                "%2, [%3];" ::"r"(su32(st + p * 8192)),
                "l"(srcA), "r"(8192), "r"(bar)
                : "memory");
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], "
                "%2, [%3];" ::"r"(su32(st + PP_A_BYTES + p * 4096)),
                "l"(srcB), "r"(4096), "r"(bar)
                : "memory");
          }
        }
        if (s == 0) last0 = c;
        else last1 = c;
      }
      // copies still in flight complete on their own; wait for them before the CTA ends
      if (last0 >= 0) wait_bar(su32(&full[0]), (uint32_t)((last0 / PP_STAGES) & 1), nullptr);
      if (last1 >= 0) wait_bar(su32(&full[1]), (uint32_t)((last1 / PP_STAGES) & 1), nullptr);
    }
  } else if (warp == 1) {
    // ---- MMA issuer
    if (lane == 0) {
      // instruction descriptor: FP32 accumulator, BF16 A and B (K-major), M 128, N set below
      const uint32_t idesc0 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(PP_M >> 4) << 24);
      for (int c = 0; c < nkc; ++c) {
        const int s = c % PP_STAGES;
        const int win = c / PP_FLUSH;
        const bool win_start = (c % PP_FLUSH) == 0;
        if (win_start && win > 0 &&
            !wait_bar(su32(&accfree), (uint32_t)((win - 1) & 1), abort)) {
          atomicExch(&abort_flag, 1);
          break;
        }
        if (!wait_bar(su32(&full[s]), (uint32_t)((c / PP_STAGES) & 1), abort)) {
          atomicExch(&abort_flag, 1);
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t stA = su32(smem + (size_t)s * PP_STAGE_BYTES);
        const uint32_t stB = stA + PP_A_BYTES;
        // slice 0 goes in three MMAs (levels 0..3, 4..5, 6..7), the others in groups of four
        // B slices; a window starts with the first two overwriting the exact levels, the
        // levels 6..7 are overwritten only by the very first MMA of the tile.  The 13 groups
        // (A slice p, first B slice q0, B slices nq) are a compile-time table, so the issue is
        // a straight sequence: descriptors are the stage's base descriptors plus constants
        // (the start-address field holds address / 16; every address stays inside the stage)
        constexpr int GP[13] = {0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 5, 6, 7};
        constexpr int GQ[13] = {0, 4, 6, 0, 4, 0, 4, 0, 4, 0, 0, 0, 0};
        constexpr int GN[13] = {4, 2, 2, 4, 3, 4, 2, 4, 1, 4, 3, 2, 1};
        const uint64_t dA = sdesc_sw64(stA), dB = sdesc_sw64(stB);
#pragma unroll
        for (int ks = 0; ks < 2; ++ks)
#pragma unroll
          for (int g = 0; g < 13; ++g) {
            const int pg = GP[g], q0 = GQ[g], nq = GN[g];
            const bool first = ks == 0 && pg == 0 && (q0 < PP_EXACT ? win_start : c == 0);
            const uint32_t acc = first ? 0u : 1u;
            const uint32_t idesc = idesc0 | ((uint32_t)((nq * PP_N) >> 3) << 17);
            const uint64_t da = dA + (uint64_t)((pg * 8192 + ks * 32) >> 4);
            const uint64_t db = dB + (uint64_t)((q0 * 4096 + ks * 32) >> 4);
            asm volatile(
                "{\n\t.reg .pred pd;\n\tsetp.ne.b32 pd, %4, 0;\n\t"
                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, pd;\n\t}" ::"r"(
                    tmem + (uint32_t)((pg + q0) * PP_N)),
                "l"(da), "l"(db), "r"(idesc), "r"(acc));
          }
        asm volatile(
            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                su32(&empty[s]))
            : "memory");
        if ((c % PP_FLUSH) == PP_FLUSH - 1 || c == nkc - 1)
          asm volatile(
              "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                  su32(&accf))
              : "memory");
      }
      // every MMA issued so far has completed before TMEM is read for the last time or freed
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              su32(&fin))
          : "memory");
      wait_bar(su32(&fin), 0u, nullptr);
    }
  } else {
    // ---- epilogue warps 2..9: TMEM lane quarter warp % 4, column half (warp - 2) / 4
    const int quarter = warp & 3, half = (warp - 2) >> 2;
    const int row = 32 * quarter + lane;
    long long T[32];
#pragma unroll
    for (int c = 0; c < 32; ++c) T[c] = 0;
    const uint32_t lane_base = tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)(32 * half);
    bool ok = true;
    for (int w = 0; w < nwin; ++w) {
      // warp-uniform decision: the TMEM loads below are .sync.aligned
      const bool got = wait_bar(su32(&accf), (uint32_t)(w & 1), abort);
      if (!__all_sync(0xffffffffu, got ? 1 : 0)) {
        atomicExch(&abort_flag, 1);
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
      for (int lv = 0; lv < PP_EXACT; ++lv) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          uint32_t v[16];
          tmem_ld16(lane_base + (uint32_t)(lv * PP_N + 16 * h), v);
#pragma unroll
          for (int t = 0; t < 16; ++t) {
            const float f = __uint_as_float(v[t]);
            const long long iv =
                (long long)__float2int_rn(f * __uint_as_float((uint32_t)(127 + 7 * lv) << 23));
            T[16 * h + t] += iv * (1LL << (7 * (PP_EXACT - 1 - lv)));
          }
        }
      }

      asm volatile("tcgen05.fence::before_thread_sync;");
      asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(&accfree)) : "memory");
    }
    if (__all_sync(0xffffffffu, (ok && !*abort) ? 1 : 0)) {
      // C = 2^(eA + eB - 14) (T 2^-35 + F), F = levels 6 + 7
      const int i = i0 + row;
      const int ei = i < a.M ? a.eA[i] + a.eshiftA : 0;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        uint32_t v6[16], v7[16];
        tmem_ld16(lane_base + (uint32_t)(6 * PP_N + 16 * h), v6);
        tmem_ld16(lane_base + (uint32_t)(7 * PP_N + 16 * h), v7);
        if constexpr (FIXED) {
          if (i < a.M) {
          // the projection iterate in fixed point: the product is (T + F 2^35) 2^(sc - 35) with
          // sc = 2 SP2_E - 14, i.e. W = T 2^8 + F 2^43 in units of 2^-55 (F rounded to an
          // integer there: an absolute 2^-56); |T| < 2^54 keeps T 2^8 exact, else the element is
          // marked out of range
          long long* W = reinterpret_cast<long long*>(a.C);
          static_assert(2 * SP2_E - 14 - 35 + SP2_FRAC == 8, "fixed-point scale of the product");
#pragma unroll
          for (int t8 = 0; t8 < 16; t8 += 8) {
            long long old[8];
#pragma unroll
            for (int t = 0; t < 8; ++t) {
              const int j = j0 + 32 * half + 16 * h + t8 + t;
              old[t] = (a.sub2 && j < a.N && i >= j) ? W[i + (size_t)j * a.ldc] : 0ll;
            }
#pragma unroll
            for (int t = 0; t < 8; ++t) {
              const int j = j0 + 32 * half + 16 * h + t8 + t;
              if (j < a.N && i >= j) {
                const long long tv = T[16 * h + t8 + t];
                const float ff = (__uint_as_float(v6[t8 + t]) + __uint_as_float(v7[t8 + t])) *
                                 0x1p43f;
                // unsigned arithmetic: wrap-around instead of undefined overflow, and the
                // out-of-range cases are replaced below
                unsigned long long w =
                    ((unsigned long long)tv << 8) + (unsigned long long)(long long)__float2int_rn(ff);
                if (a.sub2) w = 2ull * (unsigned long long)old[t] - w;
                if (tv >= (1ll << 54) || tv <= -(1ll << 54) || fabsf(ff) >= 0x1p30f ||
                    old[t] == SP2_BAD)
                  w = (unsigned long long)SP2_BAD;
                W[i + (size_t)j * a.ldc] = (long long)w;
                if (i != j) W[j + (size_t)i * a.ldc] = (long long)w;
              }
            }
          }
          }
        } else if (i < a.M) {
#pragma unroll
          for (int t = 0; t < 16; ++t) {
            const int j = j0 + 32 * half + 16 * h + t;
            if (j < a.N && !(a.sym && i < j)) {
              const double val = tile_value(T[16 * h + t], v6[t], v7[t], ei + a.eB[j] - 14);
              a.C[i + (size_t)j * a.ldc] = val;
              if (a.sym && i != j) a.C[j + (size_t)i * a.ldc] = val;
            }
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (tid == 0 && abort_flag) atomicExch(a.status, 1);
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(PP_TMEM_COLS));
}
__global__ void __launch_bounds__(PP_THREADS, 1) k_opipe(PipeArgs a) { opipe_tile(a, blockIdx.x); }

// ---- batched spectral projection on the pipe, two launches per step for every molecule of the
// list still iterating (blockIdx.y / blockIdx.z walks the molecules): kb_opipe_sq squares the
// iterate D_k from its slice image and writes D_(k+1) = D_k^2, or 2 D_k - D_k^2 (the old element
// read first), over D_k in Y; kb_sp2_slice then writes the slice image of D_(k+1) (every line
// exponent SP2_E) with the partial sums of its trace and of its squared elements, and its last
// block takes the next decision.  Molecules that left the batch or whose projection has
// converged (sp2i[0] != 0) launch nothing.
__device__ __forceinline__ int lines_padded(int n) { return ((n + PP_M - 1) / PP_M) * PP_M; }
__device__ __forceinline__ int sq_tiles(int n) {
  return ((n + PP_M - 1) / PP_M) * ((n + PP_N - 1) / PP_N);
}
// partial-sum slots of a molecule: one per block of kb_sp2_slice (8 lines)
__host__ __device__ __forceinline__ int sp2_slots(int n) {
  return ((n + PP_M - 1) / PP_M) * PP_M / 8;
}

// The decision at a new iterate D, taken by one thread after every partial sum of D is written:
// tr D in a fixed order, tr D^2 = sum of the squares of D's elements (D is symmetric) exactly in
// 128-bit integers, read past L1 since other CTAs wrote them; then the idempotency error
// tr(D - D^2), the stop test (the error no longer falls over two steps, Kruchinin, Rubensson,
// Niklasson 2016, or reaches the rounding floor) and the update D^2 or 2D - D^2 whose trace is
// closer to the occupied count (Niklasson 2002).  State: sp2i[0] converged, [1] steps taken,
// [2] update of the next step (1 square, 0 2D - D^2, -1 none), [3] pipeline status; sp2s[2..4]
// the last three idempotency errors, [4] set by a block that met an element outside the
// fixed-point range (the molecule leaves).
__device__ void sp2_decide(const MolPtrs& q, int nslots) {
  // tr D 2^55 as a signed 128-bit sum of the blocks' int64 sums, tr D^2 2^110 unsigned
  unsigned long long tlo = 0ull, slo = 0ull, shi = 0ull;
  long long thi = 0;
  for (int t = 0; t < nslots; ++t) {
    const unsigned long long* pt = q.sp2p + 3 * t;
    const long long tv = (long long)__ldcg(pt);
    tlo += (unsigned long long)tv;
    thi += (tv < 0 ? -1 : 0) + (tlo < (unsigned long long)tv ? 1 : 0);
    const unsigned long long l = __ldcg(pt + 1);
    slo += l;
    shi += __ldcg(pt + 2) + (slo < l ? 1ull : 0ull);
  }
  const double tx = ((double)thi * 0x1p64 + (double)tlo) * 0x1p-55;
  const double tx2 = ((double)shi * 0x1p64 + (double)slo) * 0x1p-110;
  const int n = q.m.nao;
  if (q.sp2i[3] != 0) {  // a tensor-core wait ran out: the molecule takes the one-molecule path
    *q.flag = -5;
    return;
  }
  if (q.sp2i[4] != 0) {  // an element outside the fixed-point range
    *q.flag = -6;
    return;
  }
  const double e = tx - tx2;
  const int k = q.sp2i[1];
  const double ekm2 = q.sp2s[3];  // after the shift below: e(k-2)
  q.sp2s[2] = q.sp2s[3];
  q.sp2s[3] = q.sp2s[4];
  q.sp2s[4] = e;
  const bool done = (k >= 2 && ekm2 < 1e-4 * n && e >= ekm2) || e <= 1e-15 * n;
  if (done) {
    q.sp2i[0] = 1;
    q.sp2i[2] = -1;
    return;
  }
  const double nocc = q.nalp;
  q.sp2i[2] = fabs(tx2 - nocc) <= fabs(2.0 * tx - tx2 - nocc) ? 1 : 0;
  q.sp2i[1] = k + 1;
}
// the last of `units` CTAs of a molecule to finish takes the decision (no separate launch):
// after the CTA's barrier one thread fences (cumulatively, the stores its barrier ordered before
// it) and counts the finished units; the CTA that completes the count decides and resets it
__device__ __forceinline__ void sp2_last_decides(const MolPtrs& q, int units) {
  __shared__ int last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(q.sp2i + 5, 1) == units - 1;
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  sp2_decide(q, units);  // one partial sum per unit
  q.sp2i[5] = 0;
}
__device__ __forceinline__ bool sq_skip(const MolPtrs& q) {
  return *q.flag < 0 || q.sp2i[0] != 0;
}
__global__ void __launch_bounds__(PP_THREADS, 1) kb_opipe_sq(const MolPtrs* __restrict__ mp,
                                                            const int* __restrict__ list) {
  const MolPtrs& q = mp[list[blockIdx.y]];
  const int n = q.m.nao;
  const int tiles = sq_tiles(n);
  if (sq_skip(q) || (int)blockIdx.x >= tiles) return;
  PipeArgs a{};
  a.A = a.B = q.img;  // a symmetric matrix: its rows are its columns
  a.eA = a.eB = q.iexp;
  a.eshiftA = 0;
  a.nlbA = a.nlbB = lines_padded(n) / 64;
  a.M = a.N = n;
  a.nkc = (n + PP_KC - 1) / PP_KC;
  a.C = q.Y;  // D_(k+1) over D_k, fixed point
  a.ldc = n;
  a.sym = 1;
  a.status = q.sp2i + 3;
  a.sub2 = q.sp2i[2] == 0 ? 1 : 0;
  a.fixed = 1;
  if (threadIdx.x == 0) {  // the tile's useful area (the upper tiles of the symmetric product exit)
    const int mt = (n + PP_M - 1) / PP_M, nt = (n + PP_N - 1) / PP_N;
    const int b = blockIdx.x, gid = b / (PP_GROUP * nt), first = gid * PP_GROUP;
    const int gsize = min(mt - first, PP_GROUP), inner = b - gid * PP_GROUP * nt;
    const int i0 = (first + inner % gsize) * PP_M, j0 = (inner / gsize) * PP_N;
    if (!(i0 + PP_M - 1 < j0))
      atomicAdd(&g_pipe_batch_flops, 2ull * (unsigned long long)min(PP_M, n - i0) *
                                         (unsigned long long)min(PP_N, n - j0) * (unsigned)n);
  }
  opipe_tile<true>(a, blockIdx.x);
}

// ---- the slice image of the iterate and the decision: each warp owns one line i of D (column i
// in memory, which equals row i), held in Y as fixed-point integers W = x 2^55; at the start
// (init) the line is D0 = (emax I - A) / (emax - emin), computed in FP64 and written to Y in
// fixed point, else it is read from Y.  Its slices (exponent SP2_E) go to img, and the line's
// diagonal element and the exact squares of its elements to the block's partial sums (exact
// integers); the last block of the molecule takes the decision.  A lane holds two neighbouring
// elements k, k + 1 of a 64-element segment (coalesced loads), so each slice plane gets one
// 32-bit word per lane.  Padding lines and positions get zero slices.
//
// Slice p of a fixed-point value Y < 2^56 is the 7-bit field a = (Y >> (49 - 7p)) & 127 (read
// from the 28-bit half that holds it); its BF16 value a 2^-7p is read off the BF16 number whose
// exponent field is 134 - 7p and mantissa field a: that number is 2^(7 - 7p) + a 2^-7p exactly,
// and subtracting 2^(7 - 7p) leaves a 2^-7p (exact: at most 7 significant bits).  Two
// elements go through one BF16x2 subtraction, and the signs go in with one OR (a zero slice of
// a negative element becomes -0, which adds nothing to a product).

// the square of Y < 2^56 as a (2^56, 2^28, 1) limb triple: Y = h 2^28 + l, Y^2 = h^2 2^56 +
// 2 h l 2^28 + l^2 (every partial product below 2^56, so per-lane sums of up to 256 stay exact)
struct Sq3 {
  unsigned long long hh = 0ull, hl = 0ull, ll = 0ull;
  __device__ __forceinline__ void add(uint32_t h, uint32_t l) {
    hh += (unsigned long long)h * h;
    hl += (unsigned long long)h * l;
    ll += (unsigned long long)l * l;
  }
  // the 128-bit value hh 2^56 + hl 2^29 + ll
  __device__ __forceinline__ void value(unsigned long long& lo, unsigned long long& hi) const {
    lo = hh << 56;
    hi = hh >> 8;
    const unsigned long long m = hl << 29, mh = hl >> 35;
    lo += m;
    hi += mh + (lo < m ? 1ull : 0ull);
    lo += ll;
    hi += (lo < ll ? 1ull : 0ull);
  }
};
__device__ __forceinline__ void add128(unsigned long long& lo, unsigned long long& hi,
                                       unsigned long long l, unsigned long long h) {
  lo += l;
  hi += h + (lo < l ? 1ull : 0ull);
}

__global__ void __launch_bounds__(256) kb_sp2_slice(const MolPtrs* __restrict__ mp,
                                                    const int* __restrict__ list, int init) {
  const MolPtrs& q = mp[list[blockIdx.z]];
  const int n = q.m.nao, lp = lines_padded(n);
  // uniform over the block; sp2i[0] changes only in the last block, after every block started
  if ((int)blockIdx.x * 8 >= lp || *q.flag < 0 || (!init && q.sp2i[0] != 0)) return;
  const int i = (int)blockIdx.x * 8 + (int)(threadIdx.x >> 5), lane = threadIdx.x & 31;
  const double emax = init ? q.sp2s[1] : 0.0, f = init ? 1.0 / (emax - q.sp2s[0]) : 0.0;
  const int nkc = (n + PP_KC - 1) / PP_KC, nlb = lp / 64;
  const size_t plane = (size_t)nlb * 2048;
  long long dw = 0;  // the line's diagonal element (an integer select per element)
  Sq3 sq;
  bool over = false;
  const double* __restrict__ am = q.A + (size_t)i * n;
  long long* __restrict__ y = reinterpret_cast<long long*>(q.Y) + (size_t)i * n;
  const bool real = i < n;
  for (int seg = 0; seg * 64 < nkc * PP_KC; ++seg) {
    const int k = seg * 64 + 2 * lane;
    if ((k >> 5) >= nkc) continue;  // the last segment may hold one chunk only
    long long w0 = 0, w1 = 0;
    if (real) {
      if (init) {  // D0 in FP64, then to fixed point (once per projection)
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          if (k + e >= n) continue;
          const double x = ((k + e == i ? emax : 0.0) - am[k + e]) * f;
          const uint64_t bits = (uint64_t)__double_as_longlong(x);
          const long long m = (long long)fixed_bits(bits, SP2_E);
          const long long w =
              ((bits >> 52) & 0x7FF) >= (uint64_t)(1023 + SP2_E) ? SP2_BAD : ((bits >> 63) ? -m : m);
          y[k + e] = w;
          (e ? w1 : w0) = w;
        }
      } else {
        if (k < n) w0 = y[k];
        if (k + 1 < n) w1 = y[k + 1];
      }
    }
    dw = k == i ? w0 : (k + 1 == i ? w1 : dw);
    // magnitudes (an out-of-range element, including the marker, counts as zero and stops the
    // molecule) and their 28-bit halves
    const unsigned long long a0 = w0 < 0 ? 0ull - (unsigned long long)w0 : (unsigned long long)w0;
    const unsigned long long a1 = w1 < 0 ? 0ull - (unsigned long long)w1 : (unsigned long long)w1;
    const bool bad0 = a0 >= (1ull << 56), bad1 = a1 >= (1ull << 56);
    over = over || bad0 || bad1;
    const unsigned long long m0 = bad0 ? 0ull : a0, m1 = bad1 ? 0ull : a1;
    const uint32_t h0 = (uint32_t)(m0 >> 28), l0 = (uint32_t)m0 & 0xFFFFFFFu;
    const uint32_t h1 = (uint32_t)(m1 >> 28), l1 = (uint32_t)m1 & 0xFFFFFFFu;
    sq.add(h0, l0);
    sq.add(h1, l1);
    const uint32_t signs = (w0 < 0 ? 0x8000u : 0u) | (w1 < 0 ? 0x80000000u : 0u);
    const size_t off = (size_t)slice_off(i, k, nlb);
    // both elements at once: 16-bit lanes hold the two elements' bits 0..15 of a half (slices
    // 3 and 2 of h, 7 and 6 of l) or its bits 14..29 (slices 1 and 0, 5 and 4); a shift and a
    // mask put a slice's 7-bit field of both elements in the lanes' mantissa fields, the
    // exponent field 134 - 7p makes each lane 2^(7-7p) + a 2^-7p exactly, and one BF16x2
    // subtraction of 2^(7-7p) leaves the packed pair of slices (exact: a has 7 bits)
    const uint32_t R[4] = {__byte_perm(h0 >> 14, h1 >> 14, 0x5410), __byte_perm(h0, h1, 0x5410),
                           __byte_perm(l0 >> 14, l1 >> 14, 0x5410), __byte_perm(l0, l1, 0x5410)};
#pragma unroll
    for (int pp = 0; pp < 8; ++pp) {
      const uint32_t bias = ((uint32_t)(134 - 7 * pp) << 7) * 0x10001u;
      const uint32_t mag = ((R[pp >> 1] >> ((pp & 1) ? 0 : 7)) & 0x007F007Fu) | bias;
      const uint32_t w = bf16x2_sub(mag, bias);
      *reinterpret_cast<uint32_t*>(q.img + off + pp * plane) = w | signs;
    }
  }
  if (init && lane == 0) q.iexp[i] = SP2_E;
  // block partial sums (exact integers): warp trees, then the warps in order
  __shared__ long long s_tr[8];
  __shared__ unsigned long long s_lo[8], s_hi[8];
  unsigned long long flo, fhi;
  sq.value(flo, fhi);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    dw += __shfl_xor_sync(0xffffffffu, dw, o);  // one lane holds the diagonal, the others 0
    add128(flo, fhi, __shfl_xor_sync(0xffffffffu, flo, o), __shfl_xor_sync(0xffffffffu, fhi, o));
  }
  over = __any_sync(0xffffffffu, over ? 1 : 0) != 0;
  if (over && lane == 0) q.sp2i[4] = 1;
  const int w = threadIdx.x >> 5;
  if (lane == 0) {
    s_tr[w] = dw;
    s_lo[w] = flo;
    s_hi[w] = fhi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    long long t = 0;  // 8 lines of |W| < 2^56: no overflow
    unsigned long long lo = 0ull, hi = 0ull;
    for (int u = 0; u < 8; ++u) {
      t += s_tr[u];
      add128(lo, hi, s_lo[u], s_hi[u]);
    }
    unsigned long long* pt = q.sp2p + 3 * blockIdx.x;
    pt[0] = (unsigned long long)t;
    pt[1] = lo;
    pt[2] = hi;
  }
  sp2_last_decides(q, lp / 8);
}

// after a projection: the converged iterate from fixed point back to FP64 in place (the products
// P = 2 X D X^T read it as doubles); every listed molecule of the projection bucket
__global__ void __launch_bounds__(256) kb_sp2_unfix(const MolPtrs* __restrict__ mp,
                                                    const int* __restrict__ list) {
  const MolPtrs& q = mp[list[blockIdx.z]];
  if (*q.flag < 0) return;
  const size_t nn = (size_t)q.m.nao * q.m.nao;
  long long* w = reinterpret_cast<long long*>(q.Y);
  for (size_t e = (size_t)blockIdx.x * 256 + threadIdx.x; e < nn; e += (size_t)gridDim.x * 256)
    q.Y[e] = w[e] == SP2_BAD ? __longlong_as_double(0x7FF8000000000000ll)
                             : (double)w[e] * 0x1p-55;
}

// ---- batched GEMM sites on the pipe (projection buckets): the rows of op(A) go into img,
// the columns of op(B) into img2, then one product per molecule
struct SiteLines {
  const double* M;
  int ld, kcontig, lines, K;
};
__device__ __forceinline__ SiteLines site_lines(const Site& s, int which) {
  if (which == 0) return {s.A, s.ld, s.ta ? 1 : 0, s.M, s.K};
  return {s.B, s.ld, s.tb ? 0 : 1, s.N, s.K};
}
// exponents of the lines: 32 lines per block (lines strided in memory) or one warp per line
// (k contiguous); grid.x covers lines_padded / 8 blocks for the widest molecule
// which operand image of a site is already split: -1 none (split it), 0 / 1 one of X's two
// cached images (rows / columns of X), 2 the projection's last iterate image in img (op(B) = D
// of X D: D is symmetric, so its columns are the lines img holds, exact for the fixed-point D)
__host__ __device__ __forceinline__ int site_ximage(int site, int which) {
  if (site == GS_FX) return which ? 1 : -1;   // B = X: its columns
  if (site == GS_XTT) return which ? -1 : 1;  // A = X^T: rows of X^T are columns of X
  if (site == GS_XD) return which ? 2 : 0;    // A = X: its rows; B = D
  if (site == GS_PXT) return which ? 0 : -1;  // B = X^T: columns of X^T are rows of X
  return -1;
}
// xdst >= 0: the image goes to X's cached image xdst instead of img (which 0) / img2 (which 1)
__global__ void __launch_bounds__(256) kb_pexp_site(const MolPtrs* __restrict__ mp,
                                                    const int* __restrict__ list, int site,
                                                    int which, int xdst) {
  const MolPtrs& q = mp[list[blockIdx.z]];
  if (*q.flag < 0) return;
  const SiteLines L = site_lines(site_of(q, site), which);
  const int lp = lines_padded(L.lines);
  int* e = xdst >= 0 ? q.xexp[xdst] : which ? q.iexp2 : q.iexp;
  if (!L.kcontig) {
    if ((int)blockIdx.x * 32 >= lp) return;
    pexp_rows_dev(L.M, L.ld, L.lines, L.K, lp, e, blockIdx.x);
    return;
  }
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (i >= lp) return;
  unsigned long long mx = 0ull;
  if (i < L.lines)
    for (int k = lane; k < L.K; k += 32) mx = max(mx, abs_bits(L.M[k + (size_t)i * L.ld]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0) e[i] = exp_of_max(mx);
}
__global__ void __launch_bounds__(256) kb_psplit_site(const MolPtrs* __restrict__ mp,
                                                      const int* __restrict__ list, int site,
                                                      int which, int xdst) {
  const MolPtrs& q = mp[list[blockIdx.z]];
  if (*q.flag < 0) return;
  const SiteLines L = site_lines(site_of(q, site), which);
  const int lp = lines_padded(L.lines), nkc = (L.K + PP_KC - 1) / PP_KC;
  if ((int)blockIdx.x >= lp / 64 || (int)blockIdx.y >= nkc) return;
  psplit_dev(L.M, L.ld, L.kcontig, L.lines, L.K, lp / 64,
             xdst >= 0 ? q.xexp[xdst] : which ? q.iexp2 : q.iexp,
             xdst >= 0 ? q.ximg[xdst] : which ? q.img2 : q.img, blockIdx.x, blockIdx.y);
}
__global__ void __launch_bounds__(PP_THREADS, 1) kb_opipe_site(const MolPtrs* __restrict__ mp,
                                                              const int* __restrict__ list,
                                                              int site) {
  const MolPtrs& q = mp[list[blockIdx.y]];
  if (*q.flag < 0) return;
  const Site s = site_of(q, site);
  const int tiles = ((s.M + PP_M - 1) / PP_M) * ((s.N + PP_N - 1) / PP_N);
  if ((int)blockIdx.x >= tiles) return;
  PipeArgs a{};
  const int xa = site_ximage(site, 0), xb = site_ximage(site, 1);
  a.A = xa >= 0 ? q.ximg[xa] : q.img;  // (xa is never 2)
  a.B = xb == 2 ? q.img : xb >= 0 ? q.ximg[xb] : q.img2;
  a.eA = xa >= 0 ? q.xexp[xa] : q.iexp;
  a.eB = xb == 2 ? q.iexp : xb >= 0 ? q.xexp[xb] : q.iexp2;
  a.eshiftA = s.alpha == 2.0 ? 1 : s.alpha == 0.5 ? -1 : 0;
  a.nlbA = lines_padded(s.M) / 64;
  a.nlbB = lines_padded(s.N) / 64;
  a.M = s.M;
  a.N = s.N;
  a.nkc = (s.K + PP_KC - 1) / PP_KC;
  a.C = s.C;
  a.ldc = s.ld;
  a.sym = s.sym ? 1 : 0;
  a.status = q.sp2i + 3;
  if (threadIdx.x == 0) {
    const int mt = (s.M + PP_M - 1) / PP_M, nt = (s.N + PP_N - 1) / PP_N;
    const int b = blockIdx.x, gid = b / (PP_GROUP * nt), first = gid * PP_GROUP;
    const int gsize = min(mt - first, PP_GROUP), inner = b - gid * PP_GROUP * nt;
    const int i0 = (first + inner % gsize) * PP_M, j0 = (inner / gsize) * PP_N;
    if (!(s.sym && i0 + PP_M - 1 < j0))
      atomicAdd(&g_pipe_batch_flops, 2ull * (unsigned long long)min(PP_M, s.M - i0) *
                                         (unsigned long long)min(PP_N, s.N - j0) * (unsigned)s.K);
  }
  opipe_tile(a, blockIdx.x);
}

}  // namespace

void pipe_site_b(const BatchLaunch& b, int site) {
  if (!b.count) return;
  static bool attr = false;
  if (!attr) {
    ck(cudaFuncSetAttribute(kb_opipe_site, cudaFuncAttributeMaxDynamicSharedMemorySize, PP_SMEM),
       "smem attr batched pipelined split gemm");
    attr = true;
  }
  const int n = b.nao_max;
  const int lp = pimage_lines(n), nkc = (n + PP_KC - 1) / PP_KC;
  const int tiles = ((n + PP_M - 1) / PP_M) * ((n + PP_N - 1) / PP_N);
  int tk = prof_kbegin(b.s);
  for (int which = 0; which < 2; ++which) {
    if (site_ximage(site, which) >= 0) continue;  // already split (X's images, the iterate)
    g_kernel_launches += 2;
    kb_pexp_site<<<dim3(lp / 8, 1, b.count), 256, 0, b.s>>>(b.mp, b.list, site, which, -1);
    kb_psplit_site<<<dim3(lp / 64, nkc, b.count), 256, 0, b.s>>>(b.mp, b.list, site, which,
                                                                   -1);
  }
  prof_kend(KS_PIPE_PREP, tk, b.s);
  ++g_kernel_launches;
  tk = prof_kbegin(b.s);
  kb_opipe_site<<<dim3(tiles, b.count), PP_THREADS, PP_SMEM, b.s>>>(b.mp, b.list, site);
  prof_kend(KS_PIPE, tk, b.s);
}

void pipe_x_images_b(const BatchLaunch& b) {
  if (!b.count) return;
  const int n = b.nao_max;
  const int lp = pimage_lines(n), nkc = (n + 31) / 32;  // split blocks of 32 k
  const int tk = prof_kbegin(b.s);
  // rows of X as op(A) of X D, columns of X as op(B) of F X
  const int src[2][2] = {{GS_XD, 0}, {GS_FX, 1}};
  for (int x = 0; x < 2; ++x) {
    g_kernel_launches += 2;
    kb_pexp_site<<<dim3(lp / 8, 1, b.count), 256, 0, b.s>>>(b.mp, b.list, src[x][0], src[x][1], x);
    kb_psplit_site<<<dim3(lp / 64, nkc, b.count), 256, 0, b.s>>>(b.mp, b.list, src[x][0],
                                                                   src[x][1], x);
  }
  prof_kend(KS_PIPE_PREP, tk, b.s);
}

// the slice image of the iterate and the next decision for every listed molecule still
// iterating (init: D0 from A and the Gershgorin bounds into Y first)
void sp2_slice_b(const BatchLaunch& b, bool init) {
  if (!b.count) return;
  const int lp = pimage_lines(b.nao_max);
  const int tk = prof_kbegin(b.s);
  ++g_kernel_launches;
  kb_sp2_slice<<<dim3(lp / 8, 1, b.count), 256, 0, b.s>>>(b.mp, b.list, init ? 1 : 0);
  prof_kend(KS_PIPE_PREP, tk, b.s);
}

// the projection iterate back to FP64 for every listed molecule (after the last step)
void sp2_unfix_b(const BatchLaunch& b) {
  if (!b.count) return;
  const size_t nn = (size_t)b.nao_max * b.nao_max;
  const int blocks = (int)std::min<size_t>((nn + 1023) / 1024, 4096);
  ++g_kernel_launches;
  kb_sp2_unfix<<<dim3(blocks, 1, b.count), 256, 0, b.s>>>(b.mp, b.list);
}

// the squaring of a projection step for every listed molecule still iterating: D^2 on the
// tensor cores from the iterate's slice image, and the next iterate (D^2 or 2D - D^2 as decided)
// over D in Y
void sp2_square_b(const BatchLaunch& b) {
  if (!b.count) return;
  static bool attr = false;
  if (!attr) {
    ck(cudaFuncSetAttribute(kb_opipe_sq, cudaFuncAttributeMaxDynamicSharedMemorySize, PP_SMEM),
       "smem attr batched pipelined split gemm");
    attr = true;
  }
  const int n = b.nao_max;
  const int tiles = ((n + PP_M - 1) / PP_M) * ((n + PP_N - 1) / PP_N);
  const int tk = prof_kbegin(b.s);
  ++g_kernel_launches;
  kb_opipe_sq<<<dim3(tiles, b.count), PP_THREADS, PP_SMEM, b.s>>>(b.mp, b.list);
  prof_kend(KS_PIPE, tk, b.s);
}

size_t pimage_bytes(int lines, int K) {
  const size_t lp = (size_t)((lines + PP_M - 1) / PP_M) * PP_M;
  const size_t kp = (size_t)((K + PP_KC - 1) / PP_KC) * PP_KC;
  return lp * kp * 8 * sizeof(uint16_t);
}
int pimage_lines(int lines) { return ((lines + PP_M - 1) / PP_M) * PP_M; }
int sp2_slot_count(int n) { return sp2_slots(n); }

// slice image of a matrix: line i, position k is M[i + k ld] (kcontig = 0: the rows of M) or
// M[k + i ld] (kcontig = 1: the columns of M); img holds pimage_bytes(lines, K) bytes and e
// pimage_lines(lines) ints
void psplit(const double* M, int ld, int kcontig, int lines, int K, PImage& img, cudaStream_t s) {
  img.lines = lines;
  img.K = K;
  const int lp = pimage_lines(lines);
  const int nkc = (K + PP_KC - 1) / PP_KC;
  g_kernel_launches += 2;
  if (kcontig) k_pexp_cols<<<(lp * 32 + 255) / 256, 256, 0, s>>>(M, ld, lines, K, lp, img.e);
  else k_pexp_rows<<<lp / 32, 256, 0, s>>>(M, ld, lines, K, lp, img.e);
  k_psplit<<<dim3(lp / 64, nkc), 256, 0, s>>>(M, ld, kcontig, lines, K, lp / 64, img.e,
                                              img.data);
}

// C = 2^eshiftA op(A) op(B) from two slice images (A.K == B.K); sym: the product is symmetric
void pgemm(const PImage& A, const PImage& B, double* C, int ldc, bool sym, int* status,
           cudaStream_t s, int eshiftA) {
  if (A.lines <= 0 || B.lines <= 0) return;
  if (A.K != B.K) throw std::runtime_error("split GEMM: inner dimensions differ");
  if (A.K > PP_KMAX) throw std::runtime_error("split GEMM: inner dimension above 12288");
  static bool attr = false;
  if (!attr) {
    ck(cudaFuncSetAttribute(k_opipe, cudaFuncAttributeMaxDynamicSharedMemorySize, PP_SMEM),
       "smem attr pipelined split gemm");
    attr = true;
  }
  PipeArgs a{};
  a.A = A.data;
  a.B = B.data;
  a.eA = A.e;
  a.eB = B.e;
  a.eshiftA = eshiftA;
  a.nlbA = pimage_lines(A.lines) / 64;
  a.nlbB = pimage_lines(B.lines) / 64;
  a.M = A.lines;
  a.N = B.lines;
  a.nkc = (A.K + PP_KC - 1) / PP_KC;
  a.C = C;
  a.ldc = ldc;
  a.sym = sym ? 1 : 0;
  a.status = status;
  const int mt = (a.M + PP_M - 1) / PP_M, nt = (a.N + PP_N - 1) / PP_N;
  g_split_flops += sym ? (unsigned long long)a.N * (a.N + 1) * A.K
                       : 2ull * a.M * a.N * A.K;
  const int tk = prof_kbegin(s);
  ++g_kernel_launches;
  k_opipe<<<mt * nt, PP_THREADS, PP_SMEM, s>>>(a);
  prof_kend(KS_GEMM, tk, s);
}

}  // namespace tb

namespace tb {
extern bool g_pipe_gemm;
}

// C = A B on the pipelined split GEMM from device pointers (column-major: A m x k with leading
// dimension m, B k x n with leading dimension k, C m x n with leading dimension m; sym: C is
// symmetric, m == n).  Allocates the two slice images for the call and synchronises the
// stream.  0 on success, 1 if a wait of the tensor-core pipeline ran out, -1 on bad arguments,
// -2 on a CUDA error.
extern "C" int tblite_gb300_split_gemm(int m, int n, int k, const double* a, const double* b,
                                       double* c, int sym, void* stream) {
  using namespace tb;
  if (m <= 0 || n <= 0 || k <= 0 || !a || !b || !c || (sym && m != n)) return -1;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  PImage ia, ib;
  int* st = nullptr;
  int hst = 0;
  int rc = 0;
  if (cudaMalloc(&ia.data, pimage_bytes(m, k)) != cudaSuccess ||
      cudaMalloc(&ia.e, sizeof(int) * pimage_lines(m)) != cudaSuccess ||
      cudaMalloc(&ib.data, pimage_bytes(n, k)) != cudaSuccess ||
      cudaMalloc(&ib.e, sizeof(int) * pimage_lines(n)) != cudaSuccess ||
      cudaMalloc(&st, sizeof(int)) != cudaSuccess) {
    rc = -2;
  } else {
    try {
      cudaMemsetAsync(st, 0, sizeof(int), s);
      psplit(a, m, 0, m, k, ia, s);
      psplit(b, k, 1, n, k, ib, s);
      pgemm(ia, ib, c, m, sym != 0, st, s);
      cudaMemcpyAsync(&hst, st, sizeof(int), cudaMemcpyDeviceToHost, s);
      if (cudaStreamSynchronize(s) != cudaSuccess) rc = -2;
      else rc = hst != 0 ? 1 : 0;
    } catch (...) {
      rc = -2;
    }
  }
  cudaFree(ia.data);
  cudaFree(ia.e);
  cudaFree(ib.data);
  cudaFree(ib.e);
  cudaFree(st);
  return rc;
}

extern "C" void tblite_gb300_set_pipelined_gemm(int enable) { tb::g_pipe_gemm = enable != 0; }

// test setting: polls of the pipelined split GEMM's pipeline waits on the current device (0:
// the default 2^22).  0 on success, -1 on a CUDA error.
extern "C" unsigned long long tblite_gb300_get_pipe_batch_flops(void) {
  unsigned long long v = 0;
  if (cudaMemcpyFromSymbol(&v, tb::g_pipe_batch_flops, sizeof(v)) != cudaSuccess) return 0;
  return v;
}

extern "C" int tblite_gb300_set_pipeline_wait_limit(int polls) {
  const int v = polls > 0 ? polls : tb::PP_WAIT;
  return cudaMemcpyToSymbol(tb::g_pipe_wait_limit, &v, sizeof(int)) == cudaSuccess ? 0 : -1;
}
