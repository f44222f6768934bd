// Split-precision GEMM engine (Ozaki scheme) on the tcgen05 tensor cores.
//
// D = alpha * op(A) * op(B) + beta * C with FP64 operands:
//  1. every row r of op(A) is scaled by 2^-ea[r] (|x| < 2^ea[r]) and cut into
//     S balanced base-2^8 digits (integers in [-128, 128], exact in bf16;
//     8S - 1 bits of the row's magnitude); every column c of op(B) likewise
//     with 2^-eb[c].  The cut is done on the FP64 bit pattern with integer
//     instructions only (no FP64 arithmetic).
//  2. for every digit pair (s, t) with s + t <= S + 1 the tensor cores form
//     the integer products P_st = A_s B_t in FP32 in tensor memory.  Pairs of
//     one level (s + t) accumulate together; a job sums a level's pairs over
//     a K range of at most 1024 terms in total, so every sum of products
//     (each at most 2^14) is below 2^24 and thus exact;
//  3. each exact partial is moved to registers and added, shifted by its
//     level, into a 64-bit integer fixed-point accumulator (integer sums: the
//     result does not depend on how terms are grouped into jobs);
//  4. one conversion to FP64 per output, scaled by 2^(ea[r] + eb[c] + ...).
// With both operands read from shared memory the tensor cores are fed at
// about 64 bytes per cycle per SM, so the cost is the number of slice-pair
// MMAs: 8-bit digits need 15 pairs for 39-bit operands where 7-bit digits
// need 21 for 42 bits.
// The GEMM kernel is warp specialized: one warp issues TMA tile loads
// (cp.async.bulk.tensor, 128B swizzle, 128 K terms per stage as two swizzle
// atoms) into a 3-stage shared-memory ring, one
// elected thread issues tcgen05.mma (M=128, N=128, K=16, bf16 -> f32) into
// two TMEM accumulators, and eight warps drain the accumulators while the next
// product accumulates.  Every wait on an mbarrier is bounded; a wait that
// gives up records a timeout in the device status word and the CTA exits.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <utility>
#include <vector>

#include "../../include/rgf.h"
#include "rgf_split.h"

namespace rgf {

namespace {

constexpr int BM = 128, BN = 128, BKE = 64;  // tile rows, cols, K elements per swizzle atom
constexpr int SBK = BKE;                      // K terms per pipeline stage (one atom)
constexpr int NSTAGE = 4;
constexpr int SPLIT_BETA = 8;
// terms per exact FP32 sum: 2^24 / 2^(2 beta - 2) (balanced digits, products <= 2^14)
constexpr int EXACT_TERMS = 1 << (24 - 2 * SPLIT_BETA + 2);
constexpr int MAXSLOTS = 24;
constexpr int MAXGROUPS = 32;
constexpr int NUM_THREADS = 320;              // warp 0 TMA, warp 1 MMA, warps 2..9 drain
constexpr uint32_t TILE_BYTES = BM * BKE * 2; // 16 KiB per operand tile (128 rows x 64 terms)
constexpr uint32_t TMEM_COLS = 512;           // two accumulators of 2 x 128 columns
constexpr unsigned long long WAIT_NS = 2000000000ull;  // 2 s bound on any mbarrier wait
constexpr unsigned char NO_SLICE = 0xFF;

// A slot is one MMA stream: digit slice s of op(A) against one or two digit
// slices of op(B) stacked along N (t1 in accumulator columns 0..127, t2 in
// 128..255), i.e. the products A_s B_t1 and A_s B_t2 of one N=256 MMA.  A
// group holds slots whose products share their levels (s + t1 = l1 for the
// first half, s + t2 = l2 for the second), so each half of the accumulator
// sums one level exactly.
struct SplitParams {
  int m, n, k;
  int S, beta, cs;
  int nslots;
  unsigned char ss[MAXSLOTS], st1[MAXSLOTS], st2[MAXSLOTS];
  // groups: slots g0 .. g0 + gs - 1 accumulate together over gchunk stages
  // at a time; level of the first half gl1, of the second gl2 (NO_SLICE: none)
  int ngroups;
  unsigned char g0[MAXGROUPS], gs[MAXGROUPS], gl1[MAXGROUPS], gl2[MAXGROUPS], gchunk[MAXGROUPS];
  int triA, triB, outLower;
  const int* exA;
  const int* exB;
  int exA_stride, exB_stride;   // per batch item (padded rows)
  const double* C;
  long long ldc, sC;
  double* D;
  long long ldd, sD;
  const double* C2;  // rows >= mD1 of C and D (at C2/D2 + r - mD1), or nullptr
  double* D2;
  int mD1;
  double alpha, betac;
  DevStatus* st;
  // Split K over ksplit CTAs per output tile (blockIdx.z = batch item *
  // ksplit + slice): slice kz runs the jobs j with j % ksplit == kz, adds its
  // fixed-point partial sums to the tile's int64 workspace with atomics
  // (integer sums: the result is the same bits whatever the order) and the
  // CTA that arrives last at the tile's counter converts, writes D and sets
  // workspace and counter back to zero.
  int ksplit;
  long long* wsk;  // 128 x 128 int64 per tile (column-major by tile column)
  int* cnt;        // arrival counter per tile
};

// ---- PTX wrappers -----------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait in the pipeline: gives up after WAIT_NS of wall time (or when
// another role of the CTA already gave up), raises the CTA abort flag,
// records a timeout in the device status word and returns false.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag,
                                          DevStatus* st) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  for (long long it = 1;; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort_flag) return false;
    if ((it & 255) == 0 && global_ns() - t0 > WAIT_NS) break;
  }
  *abort_flag = 1;
  atomicExch(&st->timeout, 1);
  return false;
}

// Bounded wait for asynchronous work this CTA itself issued (TMA loads,
// MMAs) before it may release TMEM and exit: it ignores the abort flag, so an
// aborted CTA still lets its own copies and MMAs land, and gives up only
// after WAIT_NS (recording a timeout).
__device__ __forceinline__ void mbar_wait_own(uint64_t* bar, uint32_t parity, DevStatus* st) {
  if (mbar_try_wait(bar, parity)) return;
  const unsigned long long t0 = global_ns();
  for (long long it = 1;; ++it) {
    if (mbar_try_wait(bar, parity)) return;
    if ((it & 255) == 0 && global_ns() - t0 > WAIT_NS) break;
  }
  atomicExch(&st->timeout, 1);
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar,
                                            int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// K-major operand: rows of 128 bytes, 128B swizzle, 8-row groups 1024 B apart.
// Two 128-row tiles stored back to back form one 256-row operand.
__device__ __forceinline__ uint64_t smem_desc_sw128(const void* base) {
  uint64_t d = 0;
  d |= (uint64_t)((smem_u32(base) >> 4) & 0x3FFF);       // start address
  d |= (uint64_t)1 << 16;                                 // leading byte offset (unused)
  d |= (uint64_t)(1024 >> 4) << 32;                       // stride byte offset
  d |= (uint64_t)1 << 46;                                 // descriptor version
  d |= (uint64_t)2 << 61;                                 // 128B swizzle
  return d;
}

// kind::f16 instruction descriptor: D f32, A/B bf16, both K-major, M=128, N=n.
constexpr uint32_t idesc_n(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(BM >> 4) << 24);
}
constexpr uint32_t IDESC_N128 = idesc_n(128);
constexpr uint32_t IDESC_N256 = idesc_n(256);

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                          uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// v * 2^e as the nearest double (ties to even) with integer instructions
// only -- on GB300 each FP64 warp instruction (conversions included) holds an
// SM sub-partition's FP64 unit ~76 cycles, which a 128 x 128 tile's epilogue
// would spend four times per output.  Same bits as rounding the exact value
// once, subnormal results included.
__device__ __forceinline__ double i64_ldexp(long long v, int e) {
  if (v == 0) return 0.0;
  const unsigned long long sign = v < 0 ? (1ull << 63) : 0ull;
  const unsigned long long a = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
  const int lz = __clzll((long long)a);
  int msb = 63 - lz;                               // a in [2^msb, 2^(msb + 1))
  const unsigned long long m = a << lz;            // leading one at bit 63
  unsigned long long mant = m >> 11;               // 53 significant bits
  const unsigned long long rem = m & 0x7FFull;     // the 11 bits rounded away
  if (rem > 0x400ull || (rem == 0x400ull && (mant & 1ull))) {
    ++mant;
    if (mant >> 53) {
      mant >>= 1;
      ++msb;
    }
  }
  const int E = msb + e + 1023;                    // biased exponent of the leading bit
  if (E >= 2047) return __longlong_as_double((long long)(sign | 0x7FF0000000000000ull));
  if (E <= 0) {  // below the normal range: a 2^e in units of 2^-1074, rounded
    const int t = e + 1074;
    unsigned long long q;
    if (t >= 0) {
      q = a << t;  // exact: the value is below 2^-1022
    } else if (t > -64) {
      const int r = -t;
      q = a >> r;
      const unsigned long long low = a & ((1ull << r) - 1), halfway = 1ull << (r - 1);
      if (low > halfway || (low == halfway && (q & 1ull))) ++q;
    } else {
      q = 0;
    }
    return __longlong_as_double((long long)(sign | q));
  }
  return __longlong_as_double(
      (long long)(sign | ((unsigned long long)E << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}

// exact FP32 integer partial v, weighted by 2^sh into the fixed-point sum
// (a negative sh rounds half up, as a shift of the integer)
__device__ __forceinline__ long long shifted(uint32_t bits, int sh) {
  const long long v = (long long)__float2int_rn(__uint_as_float(bits));
  return sh >= 0 ? (v << sh) : ((v + (1ll << (-sh - 1))) >> (-sh));
}

// Per-tile K range: triangular operands have no terms outside their triangle.
__device__ __forceinline__ void tile_kblocks(const SplitParams& p, int m0, int n0, int& kb_lo,
                                             int& kb_hi) {
  int lo = 0, hi = p.k;
  if (p.triA == TRI_LOWER) hi = min(hi, m0 + BM);
  if (p.triA == TRI_UPPER) lo = max(lo, m0);
  if (p.triB == TRI_LOWER) lo = max(lo, n0);
  if (p.triB == TRI_UPPER) hi = min(hi, n0 + BN);
  kb_lo = lo / SBK;
  kb_hi = hi > lo ? (hi + SBK - 1) / SBK : kb_lo;
}

// ---- the slice-product GEMM ---------------------------------------------------
// Shared memory: NSTAGE stages, each one 64-term atom of A (16 KiB) and up to
// two stacked atoms of B (32 KiB), then the barriers.
__global__ void __launch_bounds__(NUM_THREADS, 1)
    split_gemm_kernel(const __grid_constant__ CUtensorMap tmA,
                      const __grid_constant__ CUtensorMap tmB, const __grid_constant__ SplitParams p) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  uint8_t* tilesA = smem;                                  // NSTAGE x 16 KiB
  uint8_t* tilesB = smem + NSTAGE * TILE_BYTES;            // NSTAGE x 32 KiB
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + 3 * NSTAGE * TILE_BYTES);
  uint64_t* empty = full + NSTAGE;
  uint64_t* acc_full = empty + NSTAGE;                     // 2 accumulators
  uint64_t* acc_empty = acc_full + 2;
  uint64_t* mma_done = acc_empty + 2;                      // every MMA of this CTA retired
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mma_done + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  volatile int* last_flag = reinterpret_cast<volatile int*>(tmem_slot + 2);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  if (p.outLower && m0 + BM <= n0) return;  // whole tile above the diagonal (uniform exit)
  const int zb = blockIdx.z / p.ksplit;     // batch item: slice planes zb*S .. zb*S+S-1
  const int kz = blockIdx.z - zb * p.ksplit;
  const int zS = zb * p.S;

  int kb_lo, kb_hi;
  tile_kblocks(p, m0, n0, kb_lo, kb_hi);
  const int nkb = kb_hi - kb_lo;
  // jobs: for each group, K chunks of gchunk stages; this CTA runs every
  // ksplit-th of them (all of them without split K)
  int njobs_all = 0;
  for (int g = 0; g < p.ngroups; ++g)
    njobs_all += nkb > 0 ? (nkb + p.gchunk[g] - 1) / p.gchunk[g] : 0;
  const int njobs = njobs_all > kz ? (njobs_all - kz + p.ksplit - 1) / p.ksplit : 0;

  if (threadIdx.x == 0) {
    for (int s = 0; s < NSTAGE; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], 8);
    }
    mbar_init(mma_done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {  // all 512 TMEM columns: two accumulators of 256 columns
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)), "n"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;
  pdl_wait();  // the setup above overlaps the previous kernel's tail

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      long long use = 0;
      bool ok = true;
      int ja = 0;  // job index over all jobs of the tile
      for (int g = 0; g < p.ngroups && ok; ++g) {
        const int chunk = p.gchunk[g], q0 = p.g0[g], q1 = q0 + p.gs[g];
        for (int kb0 = kb_lo; kb0 < kb_hi && ok; kb0 += chunk, ++ja) {
          if (ja % p.ksplit != kz) continue;
          const int kb1 = min(kb_hi, kb0 + chunk);
          for (int q = q0; q < q1 && ok; ++q) {
            const bool two = p.st2[q] != NO_SLICE;
            for (int kb = kb0; kb < kb1; ++kb, ++use) {
              const int s = (int)(use % NSTAGE);
              const uint32_t ph = (uint32_t)((use / NSTAGE) & 1);
              if (!mbar_wait(&empty[s], ph ^ 1u, abort_flag, p.st)) { ok = false; break; }
              mbar_expect_tx(&full[s], (two ? 3 : 2) * TILE_BYTES);
              const int x = kb * SBK;  // K beyond the slices' extent reads zeros
              uint8_t* bs = tilesB + s * 2 * TILE_BYTES;
              tma_load_3d(tilesA + s * TILE_BYTES, &tmA, &full[s], x, m0, zS + p.ss[q]);
              tma_load_3d(bs, &tmB, &full[s], x, n0, zS + p.st1[q]);
              if (two) tma_load_3d(bs + TILE_BYTES, &tmB, &full[s], x, n0, zS + p.st2[q]);
            }
          }
        }
      }
      // Every stage with a load issued waits for that load to land (also on
      // abort), so no copy into this CTA's shared memory is in flight at exit.
      // Uses of one stage complete in order; only its last use can be open.
      for (int s = 0; s < NSTAGE; ++s) {
        if (use <= s) break;
        const long long last = s + ((use - 1 - s) / NSTAGE) * NSTAGE;
        mbar_wait_own(&full[s], (uint32_t)((last / NSTAGE) & 1), p.st);
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      long long use = 0;
      int j = 0;   // job index among this CTA's jobs
      int ja = 0;  // job index over all jobs of the tile
      bool ok = true;
      for (int g = 0; g < p.ngroups && ok; ++g) {
        const int chunk = p.gchunk[g], q0 = p.g0[g], q1 = q0 + p.gs[g];
        for (int kb0 = kb_lo; kb0 < kb_hi && ok; kb0 += chunk, ++ja) {
          if (ja % p.ksplit != kz) continue;
          const int kb1 = min(kb_hi, kb0 + chunk);
          const int buf = j & 1;
          const uint32_t aph = (uint32_t)((j >> 1) & 1);
          if (!mbar_wait(&acc_empty[buf], aph ^ 1u, abort_flag, p.st)) { ok = false; break; }
          tc_fence_after();
          const uint32_t tacc = tmem_base + (uint32_t)(buf * 2 * BN);
          bool first = true;
          for (int q = q0; q < q1 && ok; ++q) {
            const uint32_t idesc = p.st2[q] != NO_SLICE ? IDESC_N256 : IDESC_N128;
            for (int kb = kb0; kb < kb1; ++kb, ++use) {
              const int s = (int)(use % NSTAGE);
              const uint32_t ph = (uint32_t)((use / NSTAGE) & 1);
              if (!mbar_wait(&full[s], ph, abort_flag, p.st)) { ok = false; break; }
              tc_fence_after();
              const uint64_t ad = smem_desc_sw128(tilesA + s * TILE_BYTES);
              const uint64_t bd = smem_desc_sw128(tilesB + s * 2 * TILE_BYTES);
#pragma unroll
              for (int kk = 0; kk < BKE / 16; ++kk) {  // +32 bytes per K=16 step in the atom
                umma_bf16(tacc, ad + (uint64_t)(kk * 2), bd + (uint64_t)(kk * 2), idesc,
                          first ? 0u : 1u);
                first = false;
              }
              umma_commit(&empty[s]);  // frees the stage once these MMAs have read it
            }
          }
          if (!ok) break;
          umma_commit(&acc_full[buf]);  // accumulator ready for the drain warps
          ++j;
        }
      }
      // One more commit tracks every MMA this thread issued: wait for it (also
      // on abort) so that no MMA still writes TMEM when it is released.
      umma_commit(mma_done);
      mbar_wait_own(mma_done, 0, p.st);
    }
  } else {
    // ---------------- drain warps (2..9) ----------------
    const int q = warp & 3;            // TMEM lane quadrant this warp may access
    const int half = (warp - 2) >> 2;  // column half of the output tile: 0 or 1
    const int row = q * 32 + lane;     // accumulator row of this thread
    long long acc[64];
#pragma unroll
    for (int i = 0; i < 64; ++i) acc[i] = 0;
    int g = 0, gend = 0;  // group of job j; gend: first job index (over all jobs) after it
    for (int j = 0; j < njobs; ++j) {
      const int ja = kz + j * p.ksplit;  // index of this CTA's j-th job over all jobs
      while (ja >= gend) {
        if (gend > 0) ++g;
        gend += (nkb + p.gchunk[g] - 1) / p.gchunk[g];
      }
      const int buf = j & 1;
      if (!mbar_wait(&acc_full[buf], (uint32_t)((j >> 1) & 1), abort_flag, p.st)) break;
      tc_fence_after();
      const uint32_t taddr =
          tmem_base + ((uint32_t)(q * 32) << 16) + (uint32_t)(buf * 2 * BN + half * 64);
      const int sh1 = p.beta * (p.S - 1 - p.gl1[g]) - p.cs;
#pragma unroll
      for (int part = 0; part < 4; ++part) {
        uint32_t r[16];
        tmem_ld16(taddr + part * 16, r);
#pragma unroll
        for (int i = 0; i < 16; ++i) acc[part * 16 + i] += shifted(r[i], sh1);
      }
      if (p.gl2[g] != NO_SLICE) {
        const int sh2 = p.beta * (p.S - 1 - p.gl2[g]) - p.cs;
#pragma unroll
        for (int part = 0; part < 4; ++part) {
          uint32_t r[16];
          tmem_ld16(taddr + BN + part * 16, r);
#pragma unroll
          for (int i = 0; i < 16; ++i) acc[part * 16 + i] += shifted(r[i], sh2);
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&acc_empty[buf]);
    }
    pdl_trigger();  // the products are done: the next kernel may be scheduled
    if (p.ksplit > 1) {
      // split K: add this slice's partial sums to the tile's workspace; the
      // last slice to arrive takes the total (and leaves zeros behind)
      const long long tile =
          blockIdx.x + (long long)gridDim.x * (blockIdx.y + (long long)gridDim.y * zb);
      unsigned long long* W = reinterpret_cast<unsigned long long*>(p.wsk) + tile * (BM * BN);
      if (!*abort_flag) {
#pragma unroll
        for (int i = 0; i < 64; ++i)
          if (acc[i] != 0) atomicAdd(&W[(half * 64 + i) * BM + row], (unsigned long long)acc[i]);
      }
      __threadfence();
      asm volatile("bar.sync 1, 256;" ::: "memory");  // the eight drain warps
      if (warp == 2 && lane == 0) *last_flag = atomicAdd(&p.cnt[tile], 1) == p.ksplit - 1;
      asm volatile("bar.sync 1, 256;" ::: "memory");
      if (*last_flag) {
        __threadfence();
#pragma unroll
        for (int i = 0; i < 64; ++i) {
          unsigned long long* w = &W[(half * 64 + i) * BM + row];
          acc[i] = (long long)__ldcg(w);
          __stcg(w, 0ull);
        }
        if (warp == 2 && lane == 0) p.cnt[tile] = 0;
      }
    }
    // epilogue: every output once, v = alpha acc 2^(er + exB[c]) + beta C.
    // The accumulators go to the (now idle) pipeline shared memory and a
    // compact loop converts eight columns per pass -- the C reads of the
    // eight issued before any is used -- instead of a 64-fold unrolled body
    // (large code, slow to issue).  The columns' exponents come from two
    // coalesced loads per warp, shuffled to the lanes.  The conversion is
    // integer arithmetic (i64_ldexp): the only FP64 instruction per output is
    // the FMA with beta C.
    const int r = m0 + row;
    const bool live = r < p.m && !*abort_flag && (p.ksplit == 1 || *last_flag);
    const int t = threadIdx.x - 64;  // drain thread 0..255
    long long* eacc = reinterpret_cast<long long*>(smem);  // 64 x 256 int64 = 128 KiB
    // alpha and beta tests as integers, once (an FP64 compare per output
    // would cost as much as the FMA); alpha = -1 is a negation of the integers
    const int amode = p.alpha == 1.0 ? 0 : (p.alpha == -1.0 ? 1 : 2);
    if (!*abort_flag) {
#pragma unroll
      for (int i = 0; i < 64; ++i) eacc[i * 256 + t] = amode == 1 ? -acc[i] : acc[i];
    }
    __syncwarp();
    const int cbase = n0 + half * 64;
    const int* exBz = p.exB + (long long)zb * p.exB_stride;
    const int ex_lo = cbase + lane < p.n ? exBz[cbase + lane] : 0;
    const int ex_hi = cbase + 32 + lane < p.n ? exBz[cbase + 32 + lane] : 0;
    // every lane runs the loop (the shuffles are warp-wide); lanes without an
    // output (rows past m) only skip the loads and stores
    const bool hi = p.D2 && r >= p.mD1;
    const double* C = hi ? p.C2 + (long long)zb * p.sC - p.mD1
                         : (p.C ? p.C + (long long)zb * p.sC : nullptr);
    double* D = hi ? p.D2 + (long long)zb * p.sD - p.mD1 : p.D + (long long)zb * p.sD;
    const int er = live ? p.exA[(long long)zb * p.exA_stride + r] + p.cs - p.beta * (p.S + 1) + 2 : 0;
    const bool use_c = p.betac != 0.0;
    const double alpha = p.alpha, betac = p.betac;
    // column pointers advance by ldc / ldd (no 64-bit multiply per output:
    // on this GPU a wide integer multiply is as slow as an FP64 instruction)
    const long long ldc = p.ldc, ldd = p.ldd;
    const double* Cp = (live && use_c) ? C + r + (long long)cbase * ldc : nullptr;
    double* Dp = live ? D + r + (long long)cbase * ldd : nullptr;
    const int ncols = live ? min(64, p.n - cbase) : 0;          // columns < n
    const int cdiag = p.outLower ? r - cbase : 64;                // columns c <= r only
    const int nlive = max(0, min(ncols, cdiag + 1));
#pragma unroll 1
    for (int i0 = 0; i0 < 64; i0 += 8) {
      double cv[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        cv[q] = (Cp && i0 + q < nlive) ? *Cp : 0.0;
        if (Cp) Cp += ldc;
      }
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int i = i0 + q;
        const int ec = __shfl_sync(0xffffffffu, i < 32 ? ex_lo : ex_hi, i & 31);
        if (i < nlive) {
          double v = i64_ldexp(eacc[i * 256 + t], er + ec);
          if (amode == 2) v *= alpha;
          if (use_c) v = fma(betac, cv[q], v);
          *Dp = v;
        }
        if (Dp) Dp += ldd;
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base),
                 "n"(TMEM_COLS)
                 : "memory");
  }
}

// ---- slicing ------------------------------------------------------------------
// X is R x K with element (r, k) at X[r*rs + k*ks]; tri masks op(X)'s other
// triangle.  ex[r] = smallest e with |x| < 2^e over the row (0 for a zero row).
__device__ __forceinline__ bool tri_ok(int tri, int r, int k) {
  return tri == TRI_NONE || (tri == TRI_LOWER ? k <= r : k >= r);
}

// Balanced base-2^beta digits of x * 2^(beta*S - 1 - e) (truncated to an
// integer, |.| < 2^(beta*S - 1)): S digits, most significant first, the top
// one in [-2^(beta-1), 2^(beta-1)] and the others in [-2^(beta-1),
// 2^(beta-1) - 1], written to S planes `plane` elements apart.  With beta = 8
// every digit is exact in bf16 and every digit product is at most 2^14.
__device__ __forceinline__ void write_digits(unsigned long long bits, int e, int S, int beta,
                                             __nv_bfloat16* o, size_t plane) {
  const bool neg = (bits >> 63) != 0;
  int E = (int)((bits >> 52) & 0x7ff);
  unsigned long long mant = bits & 0xfffffffffffffull;
  if (E) mant |= 1ull << 52; else E = 1;
  const int sh = (E - 1075) + beta * S - 1 - e;
  unsigned long long xi = 0;
  if (mant != 0) {
    if (sh >= 0) xi = sh < 64 ? (mant << sh) : 0ull;
    else xi = -sh < 64 ? (mant >> (-sh)) : 0ull;
  }
  long long v = neg ? -(long long)xi : (long long)xi;
  const int half = 1 << (beta - 1), mask = (1 << beta) - 1;
  for (int s = S - 1; s > 0; --s) {
    int d = (int)v & mask;
    d -= d >= half ? mask + 1 : 0;
    v = (v - d) >> beta;
    o[(size_t)s * plane] = __float2bfloat16_rn((float)d);
  }
  o[0] = __float2bfloat16_rn((float)(int)v);
}

__device__ __forceinline__ int exp_of_max(unsigned long long mx) {
  if (mx == 0) return 0;
  const int E = (int)((mx >> 52) & 0x7ff);
  return (E == 0 ? -1022 : E - 1023) + 1;
}

// rows contiguous (rs == 1): thread per row, blockIdx.y picks a 32-term
// slice of K, partial maxima of |x| (as bit patterns) meet in atomicMax.
// Rows >= R1 are read from X2 (row r at X2 + (r - R1)) when X2 is set.
__global__ void rowmax_rowmajor_kernel(const double* X, long long ks, int R, int K, int tri,
                                       unsigned long long* mx, long long sX, int Rp,
                                       const double* X2, int R1) {
  pdl_wait();
  pdl_trigger();
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= R) return;
  X = (X2 && r >= R1 ? X2 - R1 : X) + (long long)blockIdx.z * sX;
  mx += (long long)blockIdx.z * Rp;
  const int k0 = blockIdx.y * 32, k1 = min(K, k0 + 32);
  unsigned long long m = 0;
#pragma unroll 8
  for (int k = k0; k < k1; ++k) {  // independent loads in flight
    const unsigned long long b =
        (unsigned long long)__double_as_longlong(X[r + (long long)k * ks]) & 0x7fffffffffffffffull;
    if (tri_ok(tri, r, k)) m = b > m ? b : m;
  }
  if (m) atomicMax(&mx[r], m);
}

// k contiguous (ks == 1): one warp per row
__global__ void rowmax_kmajor_kernel(const double* X, long long rs, int R, int K, int tri,
                                     unsigned long long* mx, int Rp, long long sX) {
  pdl_wait();
  pdl_trigger();
  const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (r >= Rp) return;
  X += (long long)blockIdx.y * sX;
  mx += (long long)blockIdx.y * Rp;
  unsigned long long m = 0;
  if (r < R)
    for (int k = lane; k < K; k += 32)
      if (tri_ok(tri, r, k)) {
        const unsigned long long b =
            (unsigned long long)__double_as_longlong(X[(long long)r * rs + k]) &
            0x7fffffffffffffffull;
        m = b > m ? b : m;
      }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long y = __shfl_xor_sync(0xffffffffu, m, o);
    m = y > m ? y : m;
  }
  if (lane == 0) mx[r] = m;
}

__global__ void row_exp_kernel(const unsigned long long* mx, int* ex, int Rp) {
  pdl_wait();
  pdl_trigger();
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const long long o = (long long)blockIdx.y * Rp;
  if (r < Rp) ex[o + r] = exp_of_max(mx[o + r]);
}

// 32 x 32 tiles through shared memory: read coalesced along the contiguous
// dimension, write the S digit planes coalesced along k.
// With X2 set (rs == 1 only), rows >= R1 are read from X2 + (r - R1).
__global__ void slice_kernel(const double* X, long long rs, long long ks, int R, int K, int tri,
                             const int* ex, __nv_bfloat16* out, int Rp, int Kp, int S, int beta,
                             long long sX, const double* X2, int R1) {
  __shared__ double tile[32][33];
  pdl_wait();
  pdl_trigger();
  X += (long long)blockIdx.z * sX;
  const double* Xb = X2 ? X2 - R1 + (long long)blockIdx.z * sX : X;
  ex += (long long)blockIdx.z * Rp;
  out += (size_t)blockIdx.z * S * Rp * Kp;
  const int r0 = blockIdx.y * 32, k0 = blockIdx.x * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    int rl, kl;
    if (rs == 1) { rl = tx; kl = ty + 8 * i; }
    else         { kl = tx; rl = ty + 8 * i; }
    const int r = r0 + rl, k = k0 + kl;
    double v = 0.0;
    if (r < R && k < K && tri_ok(tri, r, k))
      v = (X2 && r >= R1 ? Xb : X)[(long long)r * rs + (long long)k * ks];
    tile[rl][kl] = v;
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int rl = ty + 8 * i, r = r0 + rl, k = k0 + tx;
    if (r >= Rp || k >= Kp) continue;
    write_digits((unsigned long long)__double_as_longlong(tile[rl][tx]), r < R ? ex[r] : 0, S,
                 beta, out + (size_t)r * Kp + k, (size_t)Rp * Kp);
  }
}

// Both operands of a product with a short K in one launch: a CTA owns 32 rows
// of op(A) or op(B) (blockIdx.x below nblkA: A) and SLICE_KC terms of K
// (blockIdx.y); it finds the rows' maximum magnitudes over all of K, then
// writes the S digit planes of its K range tile by tile.
// Replaces the max / exponent / slice kernels (and the memsets) of the long-K
// path, which dominate small products.
constexpr int SLICE_KC = 128;  // K terms sliced per CTA of slice_pair_kernel

struct SliceOperand {
  const double* X;
  const double* X2;  // rows >= R1 from X2 + (r - R1) (rs == 1 only), or nullptr
  long long rs, ks, sX;
  int R, R1, Rp, tri;
  int* ex;
  __nv_bfloat16* out;
};

__global__ void __launch_bounds__(256) slice_pair_kernel(SliceOperand a, SliceOperand b, int nblkA,
                                                          int K, int Kp, int S, int beta) {
  __shared__ double tile[32][33];
  __shared__ unsigned long long red[8][33];
  pdl_wait();
  pdl_trigger();
  const bool isA = (int)blockIdx.x < nblkA;
  const SliceOperand& o = isA ? a : b;
  const int r0 = (isA ? blockIdx.x : blockIdx.x - nblkA) * 32;
  const long long z = blockIdx.z;
  const double* X = o.X + z * o.sX;
  const double* Xb = o.X2 ? o.X2 - o.R1 + z * o.sX : X;
  int* ex = o.ex + z * o.Rp;
  __nv_bfloat16* out = o.out + (size_t)z * S * o.Rp * Kp;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  auto val = [&](int r, int k) -> double {
    if (r >= o.R || k >= K || !tri_ok(o.tri, r, k)) return 0.0;
    return (o.X2 && r >= o.R1 ? Xb : X)[(long long)r * o.rs + (long long)k * o.ks];
  };
  // pass 1: row maxima of |x| as bit patterns
  if (o.rs == 1) {  // rows contiguous: lane = row, warp = k phase
    unsigned long long m = 0;
#pragma unroll 8
    for (int k = ty; k < K; k += 8) {  // independent loads in flight
      const unsigned long long v =
          (unsigned long long)__double_as_longlong(val(r0 + tx, k)) & 0x7fffffffffffffffull;
      m = v > m ? v : m;
    }
    red[ty][tx] = m;
  } else {  // k contiguous: warp = 4 rows, lane = k phase
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int rl = ty + 8 * i;
      unsigned long long m = 0;
#pragma unroll 4
      for (int k = tx; k < K; k += 32) {
        const unsigned long long v =
            (unsigned long long)__double_as_longlong(val(r0 + rl, k)) & 0x7fffffffffffffffull;
        m = v > m ? v : m;
      }
#pragma unroll
      for (int d = 16; d > 0; d >>= 1) {
        const unsigned long long y = __shfl_xor_sync(0xffffffffu, m, d);
        m = y > m ? y : m;
      }
      if (tx == 0) red[0][rl] = m;
    }
  }
  __syncthreads();
  __shared__ int exs[32];
  if (threadIdx.x < 32) {
    unsigned long long m = red[0][threadIdx.x];
    if (o.rs == 1)
      for (int w = 1; w < 8; ++w) m = red[w][threadIdx.x] > m ? red[w][threadIdx.x] : m;
    const int r = r0 + threadIdx.x;
    const int e = r < o.R ? exp_of_max(m) : 0;
    exs[threadIdx.x] = e;
    if (r < o.Rp && blockIdx.y == 0) ex[r] = e;
  }
  __syncthreads();
  // pass 2: digits, one 32 x 32 tile at a time (read along the contiguous
  // dimension, write along k)
  const size_t plane = (size_t)o.Rp * Kp;
  // this CTA's K range: SLICE_KC terms (blockIdx.y); the row maxima above span all of K
  const int kend = min(Kp, ((int)blockIdx.y + 1) * SLICE_KC);
  for (int k0 = blockIdx.y * SLICE_KC; k0 < kend; k0 += 32) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      int rl, kl;
      if (o.rs == 1) { rl = tx; kl = ty + 8 * i; }
      else           { kl = tx; rl = ty + 8 * i; }
      tile[rl][kl] = val(r0 + rl, k0 + kl);
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int rl = ty + 8 * i, r = r0 + rl, k = k0 + tx;
      if (r >= o.Rp) continue;
      write_digits((unsigned long long)__double_as_longlong(tile[rl][tx]), exs[rl], S, beta,
                   out + (size_t)r * Kp + k, plane);
    }
    __syncthreads();
  }
}

// ---- host side ------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static std::once_flag once;
  static EncodeTiledFn fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

bool make_map(CUtensorMap* map, void* base, int S, int Rp, int Kp) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)Kp, (cuuint64_t)Rp, (cuuint64_t)S};
  const cuuint64_t strides[2] = {(cuuint64_t)Kp * 2, (cuuint64_t)Kp * Rp * 2};
  const cuuint32_t box[3] = {BKE, BM, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, base, dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

constexpr size_t SMEM_BYTES = 1024 + 3 * NSTAGE * TILE_BYTES + 256;

int round_up(int x, int m) { return (x + m - 1) / m * m; }

}  // namespace

SplitEngine* SplitEngine::create(int slices, int* status) {
  *status = RGF_OK;
  if (!encode_fn()) {
    *status = RGF_ENOTSUP;
    return nullptr;
  }
  if (cudaFuncSetAttribute(split_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)SMEM_BYTES) != cudaSuccess) {
    cudaGetLastError();
    *status = RGF_ENOTSUP;
    return nullptr;
  }
  SplitEngine* e = new SplitEngine();
  e->slices_ = slices > 0 ? slices : 5;
  e->min_k_ = 64;
  return e;
}

SplitEngine::~SplitEngine() {
  device_free(ws_);
  device_free(wsk_);
}

int SplitEngine::ensure_splitk(long long tiles, cudaStream_t s) {
  if (tiles <= wsk_tiles_) return RGF_OK;
  device_free(wsk_);
  wsk_ = nullptr;
  cnt_ = nullptr;
  wsk_tiles_ = 0;
  const size_t bytes = (size_t)tiles * BM * BN * sizeof(long long) + (size_t)tiles * sizeof(int);
  void* p = nullptr;
  if (device_malloc(&p, bytes) != cudaSuccess) {
    cudaGetLastError();
    return RGF_ENOMEM;
  }
  if (cudaMemsetAsync(p, 0, bytes, s) != cudaSuccess) {  // ordered before this stream's use
    device_free(p);
    return RGF_ECUDA;
  }
  wsk_ = static_cast<long long*>(p);
  cnt_ = reinterpret_cast<int*>(wsk_ + (size_t)tiles * BM * BN);
  wsk_tiles_ = tiles;
  return RGF_OK;
}

int SplitEngine::reset_splitk(cudaStream_t s) {
  if (!wsk_) return RGF_OK;
  const size_t bytes = (size_t)wsk_tiles_ * BM * BN * sizeof(long long) +
                       (size_t)wsk_tiles_ * sizeof(int);
  return cudaMemsetAsync(wsk_, 0, bytes, s) == cudaSuccess ? RGF_OK : RGF_ECUDA;
}

int SplitEngine::ensure_ws(size_t bytes) {
  if (bytes <= ws_bytes_) return RGF_OK;
  device_free(ws_);
  ws_ = nullptr;
  ws_bytes_ = 0;
  if (device_malloc(&ws_, bytes) != cudaSuccess) {
    cudaGetLastError();
    return RGF_ENOMEM;
  }
  ws_bytes_ = bytes;
  return RGF_OK;
}

namespace {
constexpr int MAX_SLICES = 8;
constexpr int SHORT_K = 512;  // products with K up to this slice both operands in one launch
size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
// bytes of workspace one batch item of an (RpA x Kp) by (RpB x Kp) problem needs
size_t item_bytes(int S, int RpA, int RpB, int Kp) {
  return align256((size_t)S * RpA * Kp * 2) + align256((size_t)S * RpB * Kp * 2) +
         align256((size_t)(RpA + RpB) * sizeof(int)) +
         align256((size_t)(RpA + RpB) * sizeof(unsigned long long));
}

// ---- slot plan: which digit products share an MMA --------------------------
// The products A_a B_b (1-based digits a, b <= S, level a + b <= S + 1) run
// as slots (a; b1, b2): one N=256 MMA stream of A_a against B_b1 and B_b2
// stacked.  Even levels L pair with L + 1: slots (a; L - a, L + 1 - a) for
// a < L cover all of level L and all but (L, 1) of level L + 1.  The pairs
// left over, (L, 1), join the top level's product of the same a when S + 1
// is even; the rest run alone (N=128).  Per digit a this is
// ceil((S + 1 - a) / 2) slots, the fewest possible with one A digit per
// MMA: 9 slots for the 15 products of S=5, 16 for the 28 of S=7.  Slots with
// the same pair of levels form a group (one accumulator, one shift per half).
struct SlotDef {
  unsigned char s, t1, t2;  // 0-based digits; t2 = NO_SLICE: single
};
struct SlotGroup {
  unsigned char first, count, l1, l2;  // 0-based levels (s + t), l2 = NO_SLICE: single
};
struct SlotPlan {
  std::vector<SlotDef> slots;
  std::vector<SlotGroup> groups;
};

SlotPlan make_slot_plan(int S) {
  std::vector<std::array<int, 3>> raw;  // 1-based (a, b1, b2), b2 = 0: single
  std::vector<std::array<int, 2>> left, top;
  for (int L = 2; L <= S + 1; L += 2) {
    if (L + 1 <= S + 1) {
      for (int a = 1; a < L; ++a) raw.push_back({a, L - a, L + 1 - a});
      left.push_back({L, 1});  // (L, 1) of level L + 1
    } else {
      for (int a = 1; a <= S; ++a) top.push_back({a, S + 1 - a});
    }
  }
  for (const auto& l : left) {
    auto it = std::find_if(top.begin(), top.end(), [&](const std::array<int, 2>& t) {
      return t[0] == l[0] && t[1] != l[1];
    });
    if (it != top.end()) {
      raw.push_back({l[0], l[1], (*it)[1]});
      top.erase(it);
    } else {
      raw.push_back({l[0], l[1], 0});
    }
  }
  for (const auto& t : top) raw.push_back({t[0], t[1], 0});
  // group by level pair, keeping the order of first appearance
  std::vector<std::pair<int, int>> keys;
  for (const auto& r : raw) {
    const std::pair<int, int> k{r[0] + r[1] - 2, r[2] ? r[0] + r[2] - 2 : -1};
    if (std::find(keys.begin(), keys.end(), k) == keys.end()) keys.push_back(k);
  }
  SlotPlan plan;
  for (const auto& k : keys) {
    SlotGroup g{(unsigned char)plan.slots.size(), 0, (unsigned char)k.first,
                (unsigned char)(k.second < 0 ? NO_SLICE : k.second)};
    for (const auto& r : raw)
      if (r[0] + r[1] - 2 == k.first && (r[2] ? r[0] + r[2] - 2 : -1) == k.second) {
        plan.slots.push_back({(unsigned char)(r[0] - 1), (unsigned char)(r[1] - 1),
                              (unsigned char)(r[2] ? r[2] - 1 : NO_SLICE)});
        g.count++;
      }
    plan.groups.push_back(g);
  }
  return plan;
}

const SlotPlan& slot_plan(int S) {
  static const std::vector<SlotPlan> plans = [] {
    std::vector<SlotPlan> v;
    for (int s = 0; s <= MAX_SLICES; ++s) v.push_back(s ? make_slot_plan(s) : SlotPlan{});
    return v;
  }();
  return plans[S];
}

}  // namespace

int SplitEngine::reserve(int max_rows, int max_k, int batch_hint) {
  // one problem of the largest size at the largest slice count, plus room for
  // a batch of half-size problems (the top level of the batched inverses),
  // at most 1 GiB: larger batches run in chunks
  const size_t one = item_bytes(MAX_SLICES, max_rows, max_rows, max_k);
  const int h = round_up(std::max(max_k / 2, 1), BM);
  const size_t batch = (size_t)std::max(batch_hint, 1) * item_bytes(MAX_SLICES, h, h, h);
  return ensure_ws(std::max(one, std::min(batch, (size_t)1 << 30)) + 1024);
}

// Estimated device time of gemm(g) (seconds), fitted to GB300 timings of
// this kernel: about 20 us of launches, pipeline fill and epilogue, the
// slicing (about 8 us per launch plus the operands' FP64 reads and bf16
// writes at ~3 TB/s), and per wave of CTAs 120 ns per K=16 step of each MMA
// stream, divided over the split-K slices.
double SplitEngine::estimate_seconds(const GemmDesc& g, int slices) const {
  const int S = slices > 0 ? std::min(slices, MAX_SLICES) : slices_;
  const int Kp = round_up(g.k, BKE);
  const int tx = round_up(g.m, BM) / BM, ty = round_up(g.n, BN) / BN;
  long long tiles = 0;
  for (int bx = 0; bx < tx; ++bx)
    for (int by = 0; by < ty; ++by)
      if (!(g.outLower && bx * BM + BM <= by * BN)) ++tiles;
  tiles *= g.batch;
  const SlotPlan& plan = slot_plan(S);
  int jobs = 0;
  for (const SlotGroup& gr : plan.groups) {
    const int chunk = std::max(1, EXACT_TERMS / (SBK * gr.count));
    jobs += (Kp / SBK + chunk - 1) / chunk;
  }
  long long ksplit = 1;
  if (wsk_ && tiles * 2 <= num_sms_ && (long long)tx * ty * g.batch <= wsk_tiles_)
    ksplit = std::max<long long>(
        1, std::min<long long>({(long long)splitk_max_, jobs, num_sms_ / std::max(1ll, tiles)}));
  const double waves = std::ceil((double)(tiles * ksplit) / num_sms_);
  const bool same = g.A == g.B && g.lda == g.ldb && g.transA != g.transB;
  const double t_slice = (Kp <= SHORT_K ? 8e-6 : 16e-6) +
                         (g.m + (same ? 0.0 : g.n)) * (double)Kp * (8.0 + 2.0 * S) * g.batch / 3e12;
  const double steps = (double)plan.slots.size() * (Kp / 16.0) / ksplit;
  return 20e-6 + t_slice + waves * steps * 120e-9;
}

// Tensor maps are encoded once per (base, planes, rows, K) and reused: the
// workspace base is fixed per engine, so a handle's products need only a few
// distinct maps, and the driver call is a noticeable part of a product's host
// cost when stages are launched directly.
bool SplitEngine::map_for(CUtensorMap* out, void* base, int S, int Rp, int Kp) {
  const auto key = std::make_tuple(base, S, Rp, Kp);
  auto it = maps_.find(key);
  if (it != maps_.end()) {
    *out = it->second;
    return true;
  }
  if (!make_map(out, base, S, Rp, Kp)) return false;
  if (maps_.size() >= 512) maps_.clear();
  maps_.emplace(key, *out);
  return true;
}

int SplitEngine::slots(int S) {
  return S >= 1 && S <= MAX_SLICES ? (int)slot_plan(S).slots.size() : 0;
}

bool SplitEngine::supports(const GemmDesc& g) const {
  return g.k >= min_k_ && g.m > 0 && g.n > 0 && g.batch >= 1 &&
         round_up(g.m, BM) <= max_rows_ && round_up(g.n, BM) <= max_rows_ &&
         round_up(g.k, BKE) <= max_k_;
}

int SplitEngine::prepare(int max_rows, int max_k, int batch_hint, cudaStream_t s) {
  max_rows_ = round_up(std::max(max_rows, 1), BM);
  max_k_ = round_up(std::max(max_k, 1), BKE);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return RGF_ECUDA;
  }
  int st = reserve(max_rows_, max_k_, batch_hint);
  if (st) return st;
  // split K serves launches whose tiles cover at most half of the SMs
  return ensure_splitk(std::max(1, num_sms_ / 2), s);
}

long long SplitEngine::gemm(const GemmDesc& g, cudaStream_t s, DevStatus* st,
                            double* tensor_flops, int slices) {
  if (tensor_flops) *tensor_flops = 0.0;
  const int S = slices > 0 ? std::min(slices, MAX_SLICES) : slices_, beta = SPLIT_BETA;
  const int Kp = round_up(g.k, BKE);
  const int RpA = round_up(g.m, BM), RpB = round_up(g.n, BM);
  // op(B)^T is op(A) or its first n rows: the slices (and exponents) of A serve both
  const bool same = g.A == g.B && g.lda == g.ldb && g.sA == g.sB && g.transA != g.transB &&
                    g.n <= g.m && (!g.A2 || g.n <= g.mA1) && g.triA == TRI_NONE &&
                    g.triB == TRI_NONE;
  const size_t per_item = item_bytes(S, RpA, same ? 0 : RpB, Kp);
  const int chunk = (int)std::max<size_t>(1, std::min<size_t>(g.batch, ws_bytes_ / per_item));
  SplitParams p;
  std::memset(&p, 0, sizeof(p));
  p.m = g.m; p.n = g.n; p.k = g.k;
  p.S = S; p.beta = beta;
  // bound of the fixed-point accumulator: K * 2^(beta*(S+1) - 2) * 1.03 must stay below 2^62
  const double lg = std::log2((double)g.k * 1.03) + beta * (S + 1) - 2;
  p.cs = std::max(0, (int)std::ceil(lg) - 62);
  const SlotPlan& plan = slot_plan(S);
  p.nslots = (int)plan.slots.size();
  for (int q = 0; q < p.nslots; ++q) {
    p.ss[q] = plan.slots[q].s;
    p.st1[q] = plan.slots[q].t1;
    p.st2[q] = plan.slots[q].t2;
  }
  p.ngroups = (int)plan.groups.size();
  for (int gi = 0; gi < p.ngroups; ++gi) {
    const SlotGroup& gr = plan.groups[gi];
    p.g0[gi] = gr.first;
    p.gs[gi] = gr.count;
    p.gl1[gi] = gr.l1;
    p.gl2[gi] = gr.l2;
    // every half sums count * chunk * SBK products of at most 2^14: exact in FP32
    p.gchunk[gi] = (unsigned char)std::max(1, EXACT_TERMS / (SBK * gr.count));
  }
  const int np = S * (S + 1) / 2;  // digit-pair products per output tile and K term
  p.triA = g.triA; p.triB = g.triB; p.outLower = g.outLower;
  p.ldc = g.ldc; p.ldd = g.ldd; p.sC = g.sC; p.sD = g.sD;
  p.alpha = g.alpha; p.betac = g.beta;
  p.st = st;
  p.exA_stride = RpA; p.exB_stride = same ? RpA : RpB;
  const int triBt = g.triB == TRI_LOWER ? TRI_UPPER : g.triB == TRI_UPPER ? TRI_LOWER : TRI_NONE;
  long long launched = 0;
  uint8_t* base = static_cast<uint8_t*>(ws_);
  for (int b0 = 0; b0 < g.batch; b0 += chunk) {
    const int nbat = std::min(chunk, g.batch - b0);
    uint8_t* q = base;
    __nv_bfloat16* sa = reinterpret_cast<__nv_bfloat16*>(q); q += align256((size_t)nbat * S * RpA * Kp * 2);
    __nv_bfloat16* sb = same ? sa : reinterpret_cast<__nv_bfloat16*>(q);
    if (!same) q += align256((size_t)nbat * S * RpB * Kp * 2);
    int* exA = reinterpret_cast<int*>(q); q += align256((size_t)nbat * RpA * sizeof(int));
    int* exB = same ? exA : reinterpret_cast<int*>(q);
    if (!same) q += align256((size_t)nbat * RpB * sizeof(int));
    unsigned long long* mxA = reinterpret_cast<unsigned long long*>(q);
    q += align256((size_t)nbat * RpA * sizeof(unsigned long long));
    unsigned long long* mxB = reinterpret_cast<unsigned long long*>(q);
    // rows of op(X): (r, k) at X[r*rs + k*ks]; digits into out, exponents into ex
    auto slice = [&](const double* X, long long rs, long long ks, long long sX, int R, int tri,
                     int* ex, unsigned long long* mx, __nv_bfloat16* out, int Rp,
                     const double* X2 = nullptr, int R1 = 0) {
      if (rs == 1) {
        cudaMemsetAsync(mx, 0, sizeof(unsigned long long) * Rp * nbat, s);
        dim3 grid((R + 127) / 128, (g.k + 31) / 32, nbat);
        launch_k(rowmax_rowmajor_kernel, grid, dim3(128), 0, s, X, ks, R, (int)g.k, tri, mx, sX,
                 Rp, X2, R1);
      } else {
        dim3 grid((Rp * 32 + 255) / 256, nbat);
        launch_k(rowmax_kmajor_kernel, grid, dim3(256), 0, s, X, rs, R, (int)g.k, tri, mx, Rp, sX);
      }
      launch_k(row_exp_kernel, dim3((Rp + 255) / 256, nbat), dim3(256), 0, s,
               (const unsigned long long*)mx, ex, Rp);
      dim3 grid(Kp / 32, Rp / 32, nbat);
      launch_k(slice_kernel, grid, dim3(32, 8), 0, s, X, rs, ks, R, (int)g.k, tri,
               (const int*)ex, out, Rp, Kp, S, beta, sX, X2, R1);
      launched += 3;
    };
    const double* A = g.A + (long long)b0 * g.sA;
    const double* A2 = g.A2 ? g.A2 + (long long)b0 * g.sA : nullptr;
    const double* B = g.B + (long long)b0 * g.sB;
    if (Kp <= SHORT_K) {
      SliceOperand oa{A, A2, g.transA ? g.lda : 1, g.transA ? 1 : g.lda, g.sA, g.m,
                      A2 ? g.mA1 : g.m, RpA, g.triA, exA, sa};
      SliceOperand ob{B, nullptr, g.transB ? 1 : g.ldb, g.transB ? g.ldb : 1, g.sB, g.n, g.n,
                      RpB, triBt, exB, sb};
      const int nblkA = RpA / 32, nblkB = same ? 0 : RpB / 32;
      launch_k(slice_pair_kernel, dim3(nblkA + nblkB, (Kp + SLICE_KC - 1) / SLICE_KC, nbat),
               dim3(256), 0, s, oa, ob, nblkA, (int)g.k, Kp, S, beta);
      launched += 1;
    } else {
      if (!g.transA) slice(A, 1, g.lda, g.sA, g.m, g.triA, exA, mxA, sa, RpA, A2, g.mA1);
      else slice(A, g.lda, 1, g.sA, g.m, g.triA, exA, mxA, sa, RpA);
      if (!same) {
        if (!g.transB) slice(B, g.ldb, 1, g.sB, g.n, triBt, exB, mxB, sb, RpB);
        else slice(B, 1, g.ldb, g.sB, g.n, triBt, exB, mxB, sb, RpB);
      }
    }
    CUtensorMap ma, mb;
    if (!map_for(&ma, sa, S * nbat, RpA, Kp) ||
        !map_for(&mb, sb, S * nbat, same ? RpA : RpB, Kp)) {
      GemmDesc f = g;  // cannot describe the operands: FP64 kernel for this chunk
      f.batch = nbat;
      f.A = A; f.B = g.B + (long long)b0 * g.sB;
      if (g.A2) f.A2 = g.A2 + (long long)b0 * g.sA;
      if (g.C2) f.C2 = g.C2 + (long long)b0 * g.sC;
      if (g.D2) f.D2 = g.D2 + (long long)b0 * g.sD;
      f.C = g.C ? g.C + (long long)b0 * g.sC : nullptr;
      f.D = g.D + (long long)b0 * g.sD;
      launched += launch_gemm_fp64(f, s);
      continue;
    }
    p.exA = exA; p.exB = exB;
    p.C = g.C ? g.C + (long long)b0 * g.sC : nullptr;
    p.D = g.D + (long long)b0 * g.sD;
    p.C2 = g.C2 ? g.C2 + (long long)b0 * g.sC : nullptr;
    p.D2 = g.D2 ? g.D2 + (long long)b0 * g.sD : nullptr;
    p.mD1 = g.mD1;
    // split K when the output tiles fill at most half of the SMs (and the
    // workspace holds them): up to 16 slices of a tile's jobs, so that the
    // launch covers about one wave
    int ntiles = 0;
    for (int bx = 0; bx < RpA / BM; ++bx)
      for (int by = 0; by < RpB / BN; ++by)
        if (!(g.outLower && bx * BM + BM <= by * BN)) ++ntiles;
    const long long grid_tiles = (long long)(RpA / BM) * (RpB / BN) * nbat;
    p.ksplit = 1;
    if (wsk_ && (long long)ntiles * nbat * 2 <= num_sms_ && grid_tiles <= wsk_tiles_) {
      int jobs = 0;  // jobs of a tile with the full K range
      for (int gi = 0; gi < p.ngroups; ++gi) jobs += (Kp / SBK + p.gchunk[gi] - 1) / p.gchunk[gi];
      p.ksplit = std::max(1, std::min({splitk_max_, jobs, num_sms_ / (ntiles * nbat)}));
    }
    p.wsk = wsk_;
    p.cnt = cnt_;
    dim3 grid(RpA / BM, RpB / BN, nbat * p.ksplit);
    if (tensor_flops) {
      double tiles = 0.0;  // lower-only outputs skip tiles above the diagonal
      for (int bx = 0; bx < (int)grid.x; ++bx)
        for (int by = 0; by < (int)grid.y; ++by)
          if (!(g.outLower && bx * BM + BM <= by * BN)) tiles += 1.0;
      *tensor_flops += tiles * nbat * 2.0 * BM * BN * (double)round_up(Kp, SBK) * np;
    }
    launch_k(split_gemm_kernel, grid, dim3(NUM_THREADS), SMEM_BYTES, s, ma, mb, p);
    launched += 1;
  }
  return launched;
}

}  // namespace rgf
