// FP64-accurate GEMM on the BF16 tensor cores (tcgen05) for the batched SCF GEMM sites.
//
// GB300 issues FP64 at 2 lanes per clock per SM, while its BF16 tensor cores do ~3500
// multiply-adds per clock per SM.  The products of the SCF (reduction X^T F X, C = X Y, the
// densities) are therefore evaluated with the error-free splitting of Ozaki et al. (Numer.
// Algorithms 59, 2012): every row of op(A) and every column of op(B) is scaled by a power of
// two, e = ilogb(max |x|) + 1, and each element is cut into eight 7-bit integer slices,
//     x = 2^e sum_{p=1..8} a_p 2^-7p ,   a_p in [-127, 127]  (sign-magnitude, truncated at 2^-56)
// so that every slice is exact in BF16 and every slice product a_p b_q (< 2^14) is exact in the
// FP32 accumulator.  The slices are stored pre-scaled (a_p 2^-7(p-1)), so a product lands at the
// scale of its level L = p + q.  Levels 2..6 each own a TMEM accumulator whose partial sums stay
// exact integers (at most 5 products of < 2^14 over 192 values of k: < 2^24); levels 7..9 (at
// most 2^-35 of the leading level) share one accumulator; products with p + q > 9 are dropped
// (< 2^-49 of the leading level).  Every 192 values of k the exact levels are moved out of TMEM
// as integers and combined in an int64 per output element (no FP64 work); only the final value
// is converted:  C = 2^(eA + eB - 14) (T 2^-28 + V_789).  The result carries about the accuracy of
// an FP64 GEMM (the truncation and dropped terms are ~2^-49 of |A||B| per element), 36 BF16
// products replace each FP64 product.
//
// Tile: 128 x 64 outputs per CTA (one molecule per blockIdx.z), K in chunks of 32; 256 threads
// load and split the FP64 operands into shared memory (canonical K-major layout without swizzle:
// 8-row x 16-byte core matrices), one thread issues the 72 MMAs of a chunk (M = 128, N = 64,
// K = 16, kind::f16 with BF16 inputs, FP32 accumulation), commits them to an mbarrier, and all
// threads wait with an iteration limit.  TMEM: 6 accumulators x 64 columns (512 allocated); the
// 120 KB of shared memory keep one CTA per SM, so the allocation never waits on a neighbour.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>

#include "engine.h"

namespace tb {

#define BMOL const MolPtrs& q = mp[list[blockIdx.z]]
#define BARGS const MolPtrs* __restrict__ mp, const int* __restrict__ list

namespace {

constexpr int OZ_M = 128, OZ_N = 64, OZ_KC = 32, OZ_FLUSH = 6, OZ_THREADS = 256;
constexpr int OZ_TMEM_COLS = 512;
constexpr int OZ_SMEM = 120 * 1024;  // 96 KB of slices; the rest only limits residency to one CTA
constexpr int OZ_A_SLICE = OZ_M * OZ_KC;  // bf16 elements of one slice of the A tile
constexpr int OZ_B_SLICE = OZ_N * OZ_KC;

__device__ __forceinline__ double opA(const Site& s, int i, int k) {
  return s.ta ? s.A[k + (size_t)i * s.ld] : s.A[i + (size_t)k * s.ld];
}
__device__ __forceinline__ double opB(const Site& s, int k, int j) {
  return s.tb ? s.B[j + (size_t)k * s.ld] : s.B[k + (size_t)j * s.ld];
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
// shared-memory matrix descriptor: K-major, no swizzle, core matrices 128 B apart along K and
// 256 B apart along M/N (8-row groups), descriptor version 1
__device__ __forceinline__ uint64_t sdesc(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)(128 >> 4) << 16) |
         ((uint64_t)(256 >> 4) << 32) | ((uint64_t)1 << 46);
}
// BF16 bits of (-1)^sign a 2^-7p for an integer 0 <= a < 128 (exact: at most 7 significant bits)
__device__ __forceinline__ uint32_t slice_bits(uint32_t a, int p, uint32_t sign) {
  if (a == 0) return 0u;
  const uint32_t u = __float_as_uint((float)a) - ((uint32_t)(7 * p) << 23);
  return (u >> 16) | (sign << 15);
}
// the eight slices of x (|x| < 2^e), two BF16 per 32-bit word: word w of slice p holds the
// elements 2w, 2w+1 of a core row, so the caller passes the position in the row (0..7)
__device__ __forceinline__ void split_into(double x, int e, int pos, uint32_t (&w)[8][4]) {
  const uint64_t bits = (uint64_t)__double_as_longlong(x);
  const uint32_t sign = (uint32_t)(bits >> 63);
  const int ex = (int)((bits >> 52) & 0x7FF);
  uint64_t Y = 0;
  if (ex != 0) {  // zero and subnormals give zero slices
    const uint64_t m = (bits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int sh = ex - e - 1019;  // Y = |x| 2^(56 - e) < 2^56
    if (sh >= 0) Y = m << sh;
    else if (sh > -64) Y = m >> (-sh);
  }
  const int word = pos >> 1, half = (pos & 1) * 16;
#pragma unroll
  for (int p = 0; p < 8; ++p) {
    const uint32_t a = (uint32_t)(Y >> (49 - 7 * p)) & 0x7Fu;
    w[p][word] |= slice_bits(a, p, sign) << half;
  }
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (int it = 0; it < (1 << 24); ++it) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

}  // namespace

// exponent e = ilogb(max |x|) + 1 of every row of op(A) (into ex[0 .. M)) and of every column
// of op(B) (into ex[nb .. nb + N)); one warp per vector
__device__ __forceinline__ void oexp_body(const Site& s, int* ex, int nb, int v, int lane) {
  if (v < s.M) {
    double mx = 0.0;
    for (int k = lane; k < s.K; k += 32) mx = fmax(mx, fabs(opA(s, v, k)));
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) ex[v] = mx > 0.0 ? ilogb(mx) + 1 : 0;
  } else if (v - s.M < s.N && v - s.M < nb) {
    const int j = v - s.M;
    double mx = 0.0;
    for (int k = lane; k < s.K; k += 32) mx = fmax(mx, fabs(opB(s, k, j)));
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) ex[nb + j] = mx > 0.0 ? ilogb(mx) + 1 : 0;
  }
}
// batched: per molecule, the exponents go to the inverse-iteration scratch lu (free at every
// GEMM site), rows at lu[0 .. n), columns at lu[n .. 2n)
__global__ void __launch_bounds__(256) kb_oexp(BARGS, int site) {
  BMOL;
  oexp_body(site_of(q, site), reinterpret_cast<int*>(q.lu), q.m.nao,
            blockIdx.x * 8 + (threadIdx.x >> 5), threadIdx.x & 31);
}
__global__ void __launch_bounds__(256) k_oexp(Site s, int* ex) {
  oexp_body(s, ex, s.ld, blockIdx.x * 8 + (threadIdx.x >> 5), threadIdx.x & 31);
}

// one 128 x 64 output tile (i0, j0); the exponents ex: rows at ex[0 ..), columns at ex[n ..);
// returns false if the tensor-core pipeline did not answer within the wait limit
__device__ __forceinline__ bool ogemm_body(const Site& s, const int* __restrict__ ex, int i0,
                                           int j0) {
  const int n = s.ld;
  int kbeg = 0, kend = s.K;
  if (s.km == KM_LT_COLEND) kend = min(s.K, j0 + OZ_N);
  else if (s.km == KM_LT_ROWEND) kend = min(s.K, i0 + OZ_M);
  else if (s.km == KM_GE_ROWBEG) kbeg = (i0 / OZ_KC) * OZ_KC;

  extern __shared__ __align__(1024) unsigned char smem[];
  uint16_t* sA = reinterpret_cast<uint16_t*>(smem);                   // [8][2][16 groups][2][8][8]
  uint16_t* sB = reinterpret_cast<uint16_t*>(smem + 8 * OZ_A_SLICE * 2);  // [8][2][8 groups][2][8][8]
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 ::"r"(smem_u32(&tmem_base)), "r"(OZ_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_base;

  // loader roles: A core rows (row ra, k groups ga and ga + 2), B core row (row rb, group gb)
  const int ra = tid & 127, ga = tid >> 7;
  const int rb = tid & 63, gb = tid >> 6;
  const int eA = (i0 + ra < s.M) ? ex[i0 + ra] : 0;
  const int eB = (j0 + rb < s.N) ? ex[n + j0 + rb] : 0;
  // epilogue role: TMEM lane quadrant warp % 4 (row), column half warp / 4
  const int er = 32 * (warp & 3) + lane, eh = warp >> 2;
  long long T[32];
  float F[32];
#pragma unroll
  for (int c = 0; c < 32; ++c) {
    T[c] = 0;
    F[c] = 0.f;
  }
  const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(OZ_N >> 3) << 17) |
                         ((uint32_t)(OZ_M >> 4) << 24);
  uint32_t phase = 0;
  bool ok = true;
  int nchunk = 0;
  const int kc0 = (kbeg / OZ_KC) * OZ_KC;
  for (int k0 = kc0; k0 < kend; k0 += OZ_KC) {
    // ---- load and split: element (r, k) of a tile sits in slice p at
    //      p*S + (k/16)*(R*16) + (r/8)*128 + ((k%16)/8)*64 + (r%8)*8 + k%8   (bf16 units)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int g8 = ga + 2 * h;  // k group of 8 within the chunk
      uint32_t w[8][4];
#pragma unroll
      for (int p = 0; p < 8; ++p) w[p][0] = w[p][1] = w[p][2] = w[p][3] = 0u;
      const int i = i0 + ra;
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const int k = k0 + 8 * g8 + t;
        const double x = (i < s.M && k < s.K) ? opA(s, i, k) : 0.0;
        split_into(x, eA, t, w);
      }
      const int kk = 8 * g8;
      const int off = (kk / 16) * (OZ_M * 16) + (ra / 8) * 128 + ((kk % 16) / 8) * 64 + (ra % 8) * 8;
#pragma unroll
      for (int p = 0; p < 8; ++p)
        *reinterpret_cast<uint4*>(sA + p * OZ_A_SLICE + off) =
            make_uint4(w[p][0], w[p][1], w[p][2], w[p][3]);
    }
    {
      uint32_t w[8][4];
#pragma unroll
      for (int p = 0; p < 8; ++p) w[p][0] = w[p][1] = w[p][2] = w[p][3] = 0u;
      const int j = j0 + rb;
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const int k = k0 + 8 * gb + t;
        const double x = (j < s.N && k < s.K) ? opB(s, k, j) : 0.0;
        split_into(x, eB, t, w);
      }
      const int kk = 8 * gb;
      const int off = (kk / 16) * (OZ_N * 16) + (rb / 8) * 128 + ((kk % 16) / 8) * 64 + (rb % 8) * 8;
#pragma unroll
      for (int p = 0; p < 8; ++p)
        *reinterpret_cast<uint4*>(sB + p * OZ_B_SLICE + off) =
            make_uint4(w[p][0], w[p][1], w[p][2], w[p][3]);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    // ---- 72 MMAs: two k steps x 36 slice pairs (p + q <= 7, zero based)
    const bool first_in_window = (nchunk % OZ_FLUSH) == 0;
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      uint32_t fresh = first_in_window ? 0x3Fu : 0u;
#pragma unroll 1
      for (int ks = 0; ks < 2; ++ks)
#pragma unroll 1
        for (int p = 0; p < 8; ++p)
#pragma unroll 1
          for (int qq = 0; qq + p < 8; ++qq) {
            const int a = min(p + qq, 5);
            const uint32_t acc = ((fresh >> a) & 1u) ? 0u : 1u;
            fresh &= ~(1u << a);
            const uint64_t da = sdesc(smem_u32(sA + p * OZ_A_SLICE + ks * OZ_M * 16));
            const uint64_t db = sdesc(smem_u32(sB + qq * OZ_B_SLICE + ks * OZ_N * 16));
            asm volatile(
                "{\n\t.reg .pred pd;\n\tsetp.ne.b32 pd, %4, 0;\n\t"
                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, pd;\n\t}" ::"r"(
                    tmem + (uint32_t)(a * OZ_N)),
                "l"(da), "l"(db), "r"(idesc), "r"(acc));
          }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                   ::"r"(smem_u32(&mbar)) : "memory");
    }
    ok = __syncthreads_and(mbar_wait(smem_u32(&mbar), phase) ? 1 : 0) != 0;
    if (!ok) {
      // the MMAs of this chunk have not reported back: wait for them once more (bounded) so
      // that TMEM is not released under MMAs still in flight, then give up on the tile
      __syncthreads_and(mbar_wait(smem_u32(&mbar), phase) ? 1 : 0);
      asm volatile("tcgen05.fence::after_thread_sync;");
      break;
    }
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;");
    ++nchunk;
    const bool flush = (nchunk % OZ_FLUSH) == 0 || k0 + OZ_KC >= kend;
    if (flush) {
      // exact levels (a = 0..4, level a + 2) to int64, levels 7..9 to FP32
#pragma unroll
      for (int a = 0; a < 6; ++a) {
#pragma unroll
        for (int c0 = 0; c0 < 32; c0 += 8) {
          uint32_t v[8];
          const uint32_t addr = tmem + ((uint32_t)(32 * (warp & 3)) << 16) +
                                (uint32_t)(a * OZ_N + 32 * eh + c0);
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
              : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
                "=r"(v[6]), "=r"(v[7])
              : "r"(addr));
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int t = 0; t < 8; ++t) {
            const float f = __uint_as_float(v[t]);
            if (a < 5) {
              const long long iv =
                  (long long)__float2int_rn(f * __uint_as_float((uint32_t)(127 + 7 * a) << 23));
              T[c0 + t] += iv * (1LL << (7 * (4 - a)));
            } else {
              F[c0 + t] += f;
            }
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
    }
    __syncthreads();  // slices and accumulators are free for the next chunk
  }
  // ---- epilogue: C = 2^(eA + eB - 14) (T 2^-28 + F)
  if (ok) {
    const int i = i0 + er;
    if (i < s.M) {
      const int ei = ex[i];
#pragma unroll
      for (int c = 0; c < 32; ++c) {
        const int j = j0 + 32 * eh + c;
        if (j < s.N && !(s.sym && i < j)) {
          const int sc = ei + ex[n + j] - 14;
          const double scale =
              (sc > -1022 && sc < 1023) ? __hiloint2double((sc + 1023) << 20, 0) : 0.0;
          const double v = fma((double)T[c], 0x1p-28, (double)F[c]) * scale * s.alpha;
          s.C[i + (size_t)j * n] = v;
          if (s.sym && i != j) s.C[j + (size_t)i * n] = v;
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(OZ_TMEM_COLS));
  return ok;
}

__global__ void __launch_bounds__(OZ_THREADS, 1) kb_ogemm(BARGS, int site) {
  BMOL;
  const Site s = site_of(q, site);
  const int i0 = blockIdx.y * OZ_M, j0 = blockIdx.x * OZ_N;
  if (i0 >= s.M || j0 >= s.N) return;
  if (s.sym && i0 + OZ_M - 1 < j0) return;  // strictly above the diagonal: the mirror writes it
  if (*q.flag < 0) return;                  // the molecule has left the batch
  const bool ok = ogemm_body(s, reinterpret_cast<const int*>(q.lu), i0, j0);
  // the tensor-core pipeline did not answer: the molecule takes the one-molecule path
  if (!ok && threadIdx.x == 0) *q.flag = -5;
}
__global__ void __launch_bounds__(OZ_THREADS, 1) k_ogemm(Site s, const int* __restrict__ ex,
                                                         int* status) {
  const int i0 = blockIdx.y * OZ_M, j0 = blockIdx.x * OZ_N;
  if (i0 >= s.M || j0 >= s.N) return;
  if (s.sym && i0 + OZ_M - 1 < j0) return;
  const bool ok = ogemm_body(s, ex, i0, j0);
  if (!ok && threadIdx.x == 0) atomicExch(status, 1);
}

static void ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess)
    throw std::runtime_error(std::string("CUDA error '") + cudaGetErrorString(e) + "' in " + what);
}

void ogemm_b(const BatchLaunch& b, int site) {
  if (!b.count) return;
  static bool attr = false;
  if (!attr) {
    ck(cudaFuncSetAttribute(kb_ogemm, cudaFuncAttributeMaxDynamicSharedMemorySize, OZ_SMEM),
       "smem attr split gemm");
    attr = true;
  }
  const int n = b.nao_max;
  const int tk = prof_kbegin(b.s);
  g_kernel_launches += 2;
  kb_oexp<<<dim3((2 * n + 7) / 8, 1, b.count), 256, 0, b.s>>>(b.mp, b.list, site);
  kb_ogemm<<<dim3((n + OZ_N - 1) / OZ_N, (n + OZ_M - 1) / OZ_M, b.count), OZ_THREADS, OZ_SMEM,
             b.s>>>(b.mp, b.list, site);
  prof_kend(KS_GEMM, tk, b.s);
}

// one matrix product of the one-molecule path: C = op(A) op(B), all column-major with leading
// dimension ld; ex holds M + ld ints of device scratch; status is set to 1 if the tensor-core
// pipeline did not answer (checked by the caller once per single point)
void ogemm(bool ta, bool tb, int M, int N, int K, const double* A, const double* B, double* C,
           int ld, int kmode, int* ex, int* status, cudaStream_t st) {
  if (M <= 0 || N <= 0) return;
  static bool attr = false;
  if (!attr) {
    ck(cudaFuncSetAttribute(k_ogemm, cudaFuncAttributeMaxDynamicSharedMemorySize, OZ_SMEM),
       "smem attr split gemm");
    attr = true;
  }
  Site s{M, N, K, ld, A, ta, B, tb, C, kmode & 7, (kmode & KM_SYM) != 0, 1.0};
  g_split_flops += s.sym ? (unsigned long long)N * (N + 1) * K : 2ull * M * N * K;
  const int tk = prof_kbegin(st);
  g_kernel_launches += 2;
  k_oexp<<<(M + ld + 7) / 8, 256, 0, st>>>(s, ex);
  k_ogemm<<<dim3((N + OZ_N - 1) / OZ_N, (M + OZ_M - 1) / OZ_M, 1), OZ_THREADS, OZ_SMEM, st>>>(
      s, ex, status);
  prof_kend(KS_GEMM, tk, st);
}

#undef BMOL
#undef BARGS

}  // namespace tb
