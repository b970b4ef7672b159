// Mixed-precision Legendre transforms on the 5th-generation tensor cores
// (tcgen05, sm_103a): per-zonal-wavenumber batched contractions folded by
// equatorial symmetry, in split BF16 x 3 with FP32 accumulation in TMEM.
//
// A work item is (m, 128 columns c of the batch, up to 128 columns of the
// N dimension: 64 for the analysis and for tables whose tiles fit 64) and
// computes both parities p (n - m even / odd):
//   inverse  D_p[c][jj] = sum_k S_p[c][k] Pbar_p[jj][k]   (K = n index)
//            F(jn) = D_0 + D_1, F(js) = D_0 - D_1
//   forward  D_p[c][k]  = sum_jj X_p[c][jj] PW_p[k][jj]   (K = latitude pair)
//            s_{m+p+2k}^m[c] = D_p[c][k],  PW = (w/2) Pbar.
// Every operand x is split as x = hi + mid + lo (three BF16 numbers, 24
// significant bits) and the six products hi*hi, hi*mid, mid*hi, hi*lo,
// lo*hi, mid*mid are accumulated (dropped terms are below 2^-24 relative);
// hi*hi has an accumulator of its own so the small terms keep their bits.
//
// Both operands arrive by TMA (cp.async.bulk.tensor) already split into BF16
// planes and swizzled (128 B) by the tensor maps:
//   A inverse  Apack[s][c][x], K-major: written by pack_spectra_kernel from
//              the FP64 spectra (one bandwidth-bound pass, all SMs);
//   A forward  G3[s][(2m+p) Jh + jj][c], MN-major (c contiguous): written
//              split by the forward FFT;
//   B          the pre-split Pbar tiles built at plan creation.
// Warp roles (192 threads): warp 0 lane 0 issues the TMA loads of a stage
// (six boxes of A and B per 64-wide K chunk); warp 1 allocates TMEM and its
// lane 0 issues the MMAs; warps 2-5 are the epilogue (tcgen05.ld of the
// accumulators, warp w reading TMEM lanes 32 (w % 4) ..; inverse: parity
// fold, stores coalesced along c; forward: both parities through shared
// memory, stores coalesced along n).  Two shared-memory stages and two TMEM
// accumulator sets overlap loads, MMAs and epilogue of consecutive items.
// Every mbarrier wait is bounded by a globaltimer limit (1 s, knob
// "wait_limit_ms"); on expiry the kernel records an error code, stops
// issuing work, and still frees its TMEM.
#include <cuda_bf16.h>
#include <string.h>

#include "fp_conv.cuh"
#include "mbarrier.cuh"
#include "sht_plan.cuh"

namespace dccm {
namespace sht {

// Threads of a CTA: warp 0 (TMA), warp 1 (TMEM, MMA) and the epilogue
// warps, 4 (narrow shape) or 8 (wide shape: two warps per TMEM lane quarter
// share each item's epilogue).
template <bool NARROW> constexpr int tc_epi_warps() { return NARROW ? 4 : 8; }
template <bool NARROW> constexpr int tc_threads() { return 64 + 32 * tc_epi_warps<NARROW>(); }
constexpr int A_SPLIT_BYTES = 128 * 128;     // 128 rows (c) x 64 bf16 (K)
// Two shapes of the same kernel:
//   wide   (any table): two 96 KB stages (B boxes of up to 128 N rows), all
//          512 TMEM columns (two accumulator sets when they fit), one CTA
//          per SM;
//   narrow (tables whose N tiles all fit 64 rows, e.g. truncations up to
//          T85 on their Gaussian grids): one 72 KB stage (B boxes of 64
//          rows), 256 TMEM columns (one accumulator set), 90 KB of shared
//          memory in all, so two CTAs share an SM and one CTA's loads and
//          epilogue overlap the other's (a c3 launch has 172 items: one a
//          CTA instead of up to two).
template <bool NARROW> struct TcShape {
  static constexpr int NSTAGE = NARROW ? 1 : 2;
  static constexpr int B_SPLIT_BYTES = NARROW ? 64 * 128 : 128 * 128;  // N rows x 64 bf16 (K)
  static constexpr int STAGE_BYTES = 3 * A_SPLIT_BYTES + 3 * B_SPLIT_BYTES;  // 72 KB or 96 KB
  static constexpr int TMEM_COLS = NARROW ? 256 : 512;
  static constexpr int MIN_CTAS = NARROW ? 2 : 1;  // resident CTAs per SM
};
// Analysis epilogue staging: 128 rows (c) x 32 floats (16 k of both
// parities), rows padded to 33 floats (conflict-free row and column access).
constexpr int EP_LD = 33;
constexpr int EP_BYTES = 128 * EP_LD * 4;

struct MInfo {
  long long base;  // first tile row of (m, p=0)
  int nr, nq;      // rows per tile (N extent, multiple of 16), K chunks per parity
  int kv0, kv1;    // valid K per parity
  int nv0, nv1;    // valid N per parity
  int x0, x1;      // A operand coordinate of (m, p): Apack column / G3 row
  int eb;          // FP16 tables: the tiles of m hold the values times 2^eb
};

struct TcArgs {
  int dir;  // 0 inverse, 1 forward
  int N, Jh, batch;
  int ntmax;  // TMEM columns per accumulator (64 or 128)
  int brows;  // rows of this group's B boxes (64 or 128)
  int nct;    // 128-column tiles of this launch's batch
  int nacc;   // accumulator sets in TMEM (2: double buffered, 1)
  long long ncoef;
  const MInfo *mi;
  const int4 *items;  // (m, ct, nt, -)
  float *F;
  double *spec_out;
  int *err;
  int nsplit;         // operand splits: 3 (BF16 x 3) or 2 (FP16 hi + lo)
  const int *cexp;    // FP16: per field-level exponent of the A operand's scale
};

// ------------------------------------------------------------ PTX helpers
// Bounded wait: returns false (and records code) if the phase did not
// complete within the limit or another role already gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t *b, uint32_t parity, int *err, volatile int *abort_flag,
                                          int code, unsigned long long limit_ns) {
  if (mbar_try(b, parity)) return true;
  const unsigned long long t0 = gtimer();
  for (uint32_t it = 1;; ++it) {
    if (mbar_try(b, parity)) return true;
    if ((it & 255) == 0) {
      if (*abort_flag) return false;
      if (gtimer() - t0 > limit_ns) {
        *abort_flag = 1;
        atomicCAS(err, 0, code);
        return false;
      }
    }
  }
}
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
      "[%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Shared-memory operand descriptor, 128-byte swizzle, 8-row groups 1024
// bytes apart (stride byte offset).  K-major: the leading byte offset is
// unused.  MN-major: it is the distance between the 64-element (128-byte)
// column blocks along M.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;  // leading byte offset
  d |= (uint64_t)(1024 >> 4) << 32;            // stride byte offset
  d |= (uint64_t)1 << 46;                      // descriptor version (sm_100 family)
  d |= (uint64_t)2 << 61;                      // SWIZZLE_128B
  return d;
}
// kind::f16 instruction descriptor: BF16 x BF16 (bf16 = 1) or FP16 x FP16
// (bf16 = 0; A and B always of one type) -> F32, M = 128, B K-major, A
// K-major (a_mn = 0) or MN-major (a_mn = 1, bit 15).
__device__ __forceinline__ uint32_t idesc_f16kind(int n, int a_mn, int bf16) {
  const uint32_t t = bf16 ? 1u : 0u;
  return (1u << 4) | (t << 7) | (t << 10) | ((uint32_t)a_mn << 15) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(128 >> 4) << 24);
}
__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t da, uint64_t db, uint32_t idesc, int acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
      "l"(da), "l"(db), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}
// 16 consecutive TMEM columns of this thread's lane into registers, without
// waiting: several loads are issued, then one tmem_wait_ld before use.
__device__ __forceinline__ void tmem_ld16_nw(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
      "[%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
        "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
// Named barrier of the four epilogue warps (threads 64..191).
template <int NTHREADS> __device__ __forceinline__ void epi_sync() {
  asm volatile("bar.sync 1, %0;" ::"n"(NTHREADS) : "memory");
}
// 8 consecutive TMEM columns of this thread's lane, without waiting.
__device__ __forceinline__ void tmem_ld8_nw(uint32_t taddr, uint32_t (&r)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
}

// FP64 split used once per table entry at plan creation.
__device__ __forceinline__ void split3(double x, __nv_bfloat16 &h, __nv_bfloat16 &m, __nv_bfloat16 &l) {
  h = __double2bfloat16(x);
  double r = x - (double)__bfloat162float(h);
  m = __double2bfloat16(r);
  r = r - (double)__bfloat162float(m);
  l = __double2bfloat16(r);
}

// One launch covers up to MAXG truncation groups (an ensemble of mixed
// truncations): their work items are concatenated, each group with its own
// tables, tensor maps and buffers.
constexpr int MAXG = 8;
struct TcLaunch {
  CUtensorMap map[MAXG];   // B tiles
  CUtensorMap amap[MAXG];  // A operand
  TcArgs g[MAXG];
  int start[MAXG + 1];  // prefix of work items over groups
  int ngroups;
  unsigned long long wait_ns;  // limit of every mbarrier wait
  int withhold;  // 1: the load thread issues nothing (exercises the waits' expiry; nothing is in flight)
};

// Work item it -> group and (m, ct, nt); items of a group are ordered
// (m, nt, ct), heavy (small m) first, the column tiles ct of one (m, nt)
// consecutive: CTAs that run at the same time share the (m, nt) table tile
// (and the (ct, m) operand tile) in L2 instead of each fetching it from
// DRAM (a T341 table is larger than L2).
__device__ __forceinline__ void item_of(const TcArgs &a, int li, int &m, int &ct, int &nt) {
  const int4 w = a.items[li / a.nct];
  m = w.x;
  nt = w.z;
  ct = li % a.nct;
}
// The k-th work item of this CTA: rounds of gridDim.x items taken in
// alternating directions (CTA b: b, 2G-1-b, 2G+b, ...), so that with items
// heavy first the CTAs that get one item more get light ones.  Strictly
// increasing in k.
__device__ __forceinline__ int cta_item(int k) {
  const int G = (int)gridDim.x, b = (int)blockIdx.x;
  return (k & 1) ? (k + 1) * G - 1 - b : k * G + b;
}
__device__ __forceinline__ int group_of(const TcLaunch &L, int it) {
  int gi = 0;
  while (gi + 1 < L.ngroups && it >= L.start[gi + 1]) ++gi;
  return gi;
}

template <bool NARROW>
__global__ void __launch_bounds__(tc_threads<NARROW>(), TcShape<NARROW>::MIN_CTAS)
legendre_tc_kernel(const __grid_constant__ TcLaunch L) {
  using Sh = TcShape<NARROW>;
  constexpr int NSTAGE = Sh::NSTAGE, STAGE_BYTES = Sh::STAGE_BYTES, B_SPLIT_BYTES = Sh::B_SPLIT_BYTES;
  constexpr int TMEM_COLS = Sh::TMEM_COLS;
  extern __shared__ __align__(1024) unsigned char smem_dyn[];
  // 1024-byte aligned stage area (swizzle atoms are address based).
  unsigned char *sm = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(smem_dyn) + 1023) & ~(uintptr_t)1023);
  unsigned char *stage = sm;
  uint64_t *bars = reinterpret_cast<uint64_t *>(sm + NSTAGE * STAGE_BYTES);
  uint64_t *full = bars, *empty = bars + 2, *accf = bars + 4, *acce = bars + 6;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 8);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(bars + 9);

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  if (threadIdx.x == 0) {
    for (int s = 0; s < NSTAGE; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
      mbar_init(&accf[s], 1);
      mbar_init(&acce[s], 32 * tc_epi_warps<NARROW>());
    }
    *abort_flag = 0;
    mbar_init_fence();
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const int nitems = L.start[L.ngroups];
  if (warp == 0 && lane < 2 * L.ngroups) {  // descriptors into the TMA unit's cache, behind the previous kernel
    const CUtensorMap *mp = (lane & 1) ? &L.amap[lane >> 1] : &L.map[lane >> 1];
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(mp)) : "memory");
  }
  if (warp == 2 && lane < 2) {
    // The item list and MInfo of this CTA's first two items (plan constants,
    // not written by the previous kernel) into L1 while the previous kernel
    // finishes: every role reads them right after the dependency wait.
    const int it = cta_item(lane);
    if (it < nitems) {
      const int gi = group_of(L, it);
      int m, ct, nt;
      item_of(L.g[gi], it - L.start[gi], m, ct, nt);
      const char *q = reinterpret_cast<const char *>(L.g[gi].mi + m);
      asm volatile("prefetch.global.L1 [%0];" ::"l"(q));
      asm volatile("prefetch.global.L1 [%0];" ::"l"(q + sizeof(MInfo) - 1));
    }
  }
  pdl_wait();  // the operands come from the previous kernel (pack or forward FFT)
  pdl_trigger();

  if (warp == 0) {
    // ---------------------------------------------------------- TMA
    if (lane == 0 && !L.withhold) {
      int g = 0;  // chunk counter
      bool ok = true;
      for (int k = 0, it = cta_item(0); it < nitems && ok; it = cta_item(++k)) {
        const int gi = group_of(L, it);
        const TcArgs &a = L.g[gi];
        int m, ct, nt;
        item_of(a, it - L.start[gi], m, ct, nt);
        const MInfo mi = a.mi[m];
        for (int p = 0; p < 2 && ok; ++p) {
          const int kv = p ? mi.kv1 : mi.kv0;
          const int nq = (kv + 63) / 64;
          const int x0 = p ? mi.x1 : mi.x0;
          for (int q = 0; q < nq; ++q, ++g) {
            const int s = g % NSTAGE;
            if (!mbar_wait(&empty[s], ((g / NSTAGE) & 1) ^ 1, a.err, abort_flag, 1, L.wait_ns)) { ok = false; break; }
            unsigned char *As = stage + s * STAGE_BYTES;
            unsigned char *Bs = As + 3 * A_SPLIT_BYTES;
            mbar_arrive_tx(&full[s], (uint32_t)(a.nsplit * (A_SPLIT_BYTES + a.brows * 128)));
            for (int sp = 0; sp < a.nsplit; ++sp) {
              unsigned char *Ad = As + sp * A_SPLIT_BYTES;
              if (a.dir == 0) {
                tma_load_3d(Ad, &L.amap[gi], x0 + 64 * q, ct * 128, sp, &full[s]);
              } else {
                tma_load_3d(Ad, &L.amap[gi], ct * 128, x0 + 64 * q, sp, &full[s]);
                tma_load_3d(Ad + 8192, &L.amap[gi], ct * 128 + 64, x0 + 64 * q, sp, &full[s]);
              }
              const long long row0 = mi.base + ((long long)(p * mi.nq + q) * a.nsplit + sp) * mi.nr + nt * a.brows;
              tma_load_2d(Bs + sp * B_SPLIT_BYTES, &L.map[gi], 0, (int)row0, &full[s]);
            }
          }
        }
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    // ------------------------------------------------------------- MMA
    if (lane == 0) {
      int g = 0, li = 0;
      bool ok = true;
      for (int it = cta_item(0); it < nitems && ok; it = cta_item(++li)) {
        const int gi = group_of(L, it);
        const TcArgs &a = L.g[gi];
        int m, ct, nt;
        item_of(a, it - L.start[gi], m, ct, nt);
        const MInfo mi = a.mi[m];
        const int nrow = min(a.brows, mi.nr - nt * a.brows);
        const int amn = a.dir;  // forward A is MN-major
        const uint32_t idesc = idesc_f16kind(nrow, amn, a.nsplit == 3);
        const int ncross = a.nsplit == 3 ? 5 : 2;
        const int ab = a.nacc == 2 ? (li & 1) : 0;
        const int ar = a.nacc == 2 ? (li >> 1) : li;  // use count of this accumulator set
        if (!mbar_wait(&acce[ab], (ar & 1) ^ 1, a.err, abort_flag, 2, L.wait_ns)) { ok = false; break; }
        tc_fence_after();
        for (int p = 0; p < 2 && ok; ++p) {
          const int kv = p ? mi.kv1 : mi.kv0;
          const int nq = (kv + 63) / 64;
          const uint32_t dmain = tmem + ab * 4 * a.ntmax + (p * 2) * a.ntmax;
          const uint32_t dcross = dmain + a.ntmax;
          int accm = 0, accx = 0;
          for (int q = 0; q < nq; ++q, ++g) {
            const int s = g % NSTAGE;
            if (!mbar_wait(&full[s], (g / NSTAGE) & 1, a.err, abort_flag, 3, L.wait_ns)) { ok = false; break; }
            tc_fence_after();
            const uint32_t As = smem_u32(stage + s * STAGE_BYTES);
            const uint32_t Bs = As + 3 * A_SPLIT_BYTES;
            const int ksteps = min(4, (kv - q * 64 + 15) / 16);
            for (int ks = 0; ks < ksteps; ++ks) {
              // K step of 16: 32 bytes along a K-major row, 16 rows of an MN-major tile
              const uint32_t ka = amn ? ks * 2048 : ks * 32;
              const uint32_t lbo = amn ? 8192 : 16;
              const uint32_t kb = ks * 32;
              mma_bf16(dmain, smem_desc(As + ka, lbo), smem_desc(Bs + kb, 16), idesc, accm);
              accm = 1;
              // (A split, B split): BF16 x 3 hi*mid, mid*hi, hi*lo, lo*hi,
              // mid*mid; FP16 hi + lo: hi*lo, lo*hi
              const int pa[5] = {0, 1, 0, 2, 1};
              const int pb[5] = {1, 0, 2, 0, 1};
#pragma unroll
              for (int u = 0; u < 5; ++u) {
                if (u < ncross) {
                  mma_bf16(dcross, smem_desc(As + pa[u] * A_SPLIT_BYTES + ka, lbo),
                           smem_desc(Bs + pb[u] * B_SPLIT_BYTES + kb, 16), idesc, accx);
                  accx = 1;
                }
              }
            }
            mma_commit(&empty[s]);
          }
        }
        mma_commit(&accf[ab]);
      }
    }
    __syncwarp();
  } else {
    // -------------------------------------------------------- epilogue
    constexpr int EW = tc_epi_warps<NARROW>(), EH = EW / 4, ET = 32 * EW;
    const int quad = warp & 3;             // TMEM lane quarter this warp may read
    const int widx = warp - 2;             // 0 .. EW-1
    const int half = widx >> 2;            // 0 .. EH-1: which share of the quarter's columns
    const int row = quad * 32 + lane;
    float *ep = reinterpret_cast<float *>(sm + NSTAGE * STAGE_BYTES + 128);  // [128][EP_LD]
    int li = 0;
    // A failed wait ends the inverse epilogue; the forward epilogue's warps
    // keep passing their shared barriers (without TMEM loads or stores) so
    // that none of them waits on a warp that left.
    bool dead = false;
    for (int it = cta_item(0); it < nitems; it = cta_item(++li)) {
      const int gi = group_of(L, it);
      const TcArgs &a = L.g[gi];
      int m, ct, nt;
      item_of(a, it - L.start[gi], m, ct, nt);
      const int C2B = 2 * a.batch;
      const MInfo mi = a.mi[m];
      const int nrow = min(a.brows, mi.nr - nt * a.brows);
      const int ab = a.nacc == 2 ? (li & 1) : 0;
      const int ar = a.nacc == 2 ? (li >> 1) : li;
      if (dead || !mbar_wait(&accf[ab], ar & 1, a.err, abort_flag, 4, L.wait_ns)) {
        dead = true;
        if (a.dir == 0) break;
      }
      tc_fence_after();
      const int c = ct * 128 + row;
      const int NT = a.ntmax;
      const uint32_t tbase = tmem + ((uint32_t)(quad * 32) << 16) + ab * 4 * NT;
      // FP16 operands were scaled by 2^(14 - cexp) (spectra) or 2^(13 - cexp)
      // (Fourier coefficients) and 2^eb (tables): undo both (exact)
      float us = 1.f;
      if (a.nsplit == 2 && c < C2B) us = pow2f((a.dir ? 13 : 14) * -1 + a.cexp[c >> 1] - mi.eb);
      if (a.dir == 0) {
        const int J = 2 * a.Jh;
        const bool odd = mi.kv1 > 0;
        for (int j0 = 16 * half; j0 < nrow; j0 += 16 * EH) {
          // the four accumulators' columns j0..j0+15, one wait for all
          uint32_t re[16], rx[16], ro[16], ry[16];
          tmem_ld16_nw(tbase + j0, re);
          tmem_ld16_nw(tbase + NT + j0, rx);
          if (odd) {
            tmem_ld16_nw(tbase + 2 * NT + j0, ro);
            tmem_ld16_nw(tbase + 3 * NT + j0, ry);
          }
          tmem_wait_ld();
          float e[16], o[16];
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            e[i] = __uint_as_float(re[i]) + __uint_as_float(rx[i]);
            o[i] = odd ? __uint_as_float(ro[i]) + __uint_as_float(ry[i]) : 0.f;
          }
          if (c < C2B) {
#pragma unroll
            for (int i = 0; i < 16; ++i) {
              const int jj = nt * a.brows + j0 + i;
              if (jj < a.Jh) {
                a.F[((long long)m * J + (a.Jh + jj)) * C2B + c] = (e[i] + o[i]) * us;
                a.F[((long long)m * J + (a.Jh - 1 - jj)) * C2B + c] = (e[i] - o[i]) * us;
              }
            }
          }
        }
      } else {
        // Columns k0..k0+15 of both parities go to shared memory as
        // [c][2i + p] (coefficient n = nbase + 2 k0 + 2i + p), then warp w
        // writes the contiguous runs of n of field-levels w, w + 4, ...:
        // 16-byte stores of consecutive coefficients.
        float *erow = ep + row * EP_LD;
        const int nbase = m + 2 * nt * a.brows;
        for (int k0 = 0; k0 < nrow; k0 += 16) {
          if (nt * a.brows + k0 >= mi.nv0) break;  // nv0 >= nv1; uniform over the epilogue warps
          if (!dead) {
            if constexpr (EH == 1) {
              uint32_t r0[16], x0[16], r1[16], x1[16];
              tmem_ld16_nw(tbase + k0, r0);
              tmem_ld16_nw(tbase + NT + k0, x0);
              tmem_ld16_nw(tbase + 2 * NT + k0, r1);
              tmem_ld16_nw(tbase + 3 * NT + k0, x1);
              tmem_wait_ld();
#pragma unroll
              for (int i = 0; i < 16; ++i) {
                erow[2 * i] = (__uint_as_float(r0[i]) + __uint_as_float(x0[i])) * us;
                erow[2 * i + 1] = (__uint_as_float(r1[i]) + __uint_as_float(x1[i])) * us;
              }
            } else {  // two warps a quarter: columns k0 + 8 half .. + 7 each
              const int k8 = k0 + 8 * half;
              uint32_t r0[8], x0[8], r1[8], x1[8];
              tmem_ld8_nw(tbase + k8, r0);
              tmem_ld8_nw(tbase + NT + k8, x0);
              tmem_ld8_nw(tbase + 2 * NT + k8, r1);
              tmem_ld8_nw(tbase + 3 * NT + k8, x1);
              tmem_wait_ld();
#pragma unroll
              for (int i = 0; i < 8; ++i) {
                erow[2 * (8 * half + i)] = (__uint_as_float(r0[i]) + __uint_as_float(x0[i])) * us;
                erow[2 * (8 * half + i) + 1] = (__uint_as_float(r1[i]) + __uint_as_float(x1[i])) * us;
              }
            }
          }
          epi_sync<ET>();
          const int n = nbase + 2 * k0 + lane;
          if (!dead && n <= a.N) {
            double2 *dst = reinterpret_cast<double2 *>(a.spec_out) + idx_mn(a.N, m, n);
            for (int bl = widx; bl < 64; bl += EW) {
              const int c0 = ct * 128 + 2 * bl;
              if (c0 >= C2B) break;
              const double re = f32_to_f64(ep[2 * bl * EP_LD + lane]);
              const double im = m == 0 ? 0.0 : f32_to_f64(ep[(2 * bl + 1) * EP_LD + lane]);
              dst[(long long)(c0 >> 1) * a.ncoef] = make_double2(re, im);
            }
          }
          epi_sync<ET>();
        }
      }
      tc_fence_before();
      mbar_arrive(&acce[ab]);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS)
                 : "memory");
  }
}

// ------------------------------------------------------------ spectra pack
// Apack[s][2b + comp][x] = split s of the FP32 rounding of the spectral
// coefficient of field-level b at column x of its (m, p) segment.  A unit
// is 16 consecutive coefficients n = n0 .. n0 + 15 (n0 = m + 16 q) of one m,
// i.e. columns 8q .. 8q + 7 of both parities' segments; one thread per
// (field-level, unit, parity).  A unit's two threads read the interleaved
// halves of one contiguous 256-byte run of the spectra (a warp's units are
// neighbouring runs); each of a thread's stores is one 16-byte run of a
// segment.  A segment of c coefficients is 16 ceil(c /
// 16) columns long; a run is written only if it starts below c (then it
// ends inside the segment; its entries past N are written as 0), and the
// columns no run reaches stay zero from plan creation.
struct PackGroup {
  const double2 *spec;
  const int4 *units;  // (m, q, x of parity 0, x of parity 1)
  unsigned short *A;
  long long ncoef, KX;
  long long t0;       // first thread of this group; nunits threads per field-level
  int nunits, N, C2Bp, batch;
  int nsplit;         // 3: BF16 x 3; 2: FP16 hi + lo scaled by 2^(14 - cexp[b])
  const int *cexp;    // FP16: exponent of the field-level's largest |coefficient|
};
struct PackLaunch {
  PackGroup g[MAXG];
  int ngroups;
  long long total;
};

__global__ void __launch_bounds__(128) pack_spectra_kernel(const __grid_constant__ PackLaunch L) {
  pdl_wait();  // Apack is read by the previous step's synthesis
  pdl_trigger();
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= L.total) return;
  int gi = 0;
  while (gi + 1 < L.ngroups && t >= L.g[gi + 1].t0) ++gi;
  const PackGroup &G = L.g[gi];
  // thread = (field-level, unit, parity), parity fastest: the two threads of
  // a unit read the interleaved halves of one 256-byte run
  const long long u2 = t - G.t0;
  const int b = (int)(u2 / (2 * G.nunits));
  const int r = (int)(u2 - (long long)b * 2 * G.nunits);
  const int p = r & 1;
  const int4 w = __ldg(G.units + (r >> 1));
  const int m = w.x, n0 = m + 16 * w.y;
  // columns 8q .. 8q+7 of this parity hold at least one coefficient, else
  // the run lies past the segment (whose rounded length covers every run
  // that starts inside it) and is not written
  if (8 * w.y >= count_np(G.N, m, p)) return;
  const double2 *src = G.spec + (size_t)b * G.ncoef + idx_mn(G.N, m, n0) + p;
  double2 v[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) v[j] = n0 + p + 2 * j <= G.N ? __ldg(src + 2 * j) : make_double2(0.0, 0.0);
  const size_t plane = (size_t)G.C2Bp * G.KX;
  const int sc = G.nsplit == 2 ? 14 - G.cexp[b] : 0;
#pragma unroll
  for (int comp = 0; comp < 2; ++comp) {
    unsigned short *o = G.A + (size_t)(2 * b + comp) * G.KX + (p ? w.w : w.z);
    float f[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const double x = comp ? v[j].y : v[j].x;
      f[j] = f64_to_f32_rn_z(G.nsplit == 2 ? scale_pow2(x, sc) : x);
    }
    if (G.nsplit == 2) {
      unsigned h[4], l[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) split2h_x2(make_float2(f[2 * i], f[2 * i + 1]), h[i], l[i]);
      *reinterpret_cast<uint4 *>(o) = make_uint4(h[0], h[1], h[2], h[3]);
      *reinterpret_cast<uint4 *>(o + plane) = make_uint4(l[0], l[1], l[2], l[3]);
    } else {
      unsigned h[4], md[4], l[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) split3f_x2(make_float2(f[2 * i], f[2 * i + 1]), h[i], md[i], l[i]);
      *reinterpret_cast<uint4 *>(o) = make_uint4(h[0], h[1], h[2], h[3]);
      *reinterpret_cast<uint4 *>(o + plane) = make_uint4(md[0], md[1], md[2], md[3]);
      *reinterpret_cast<uint4 *>(o + 2 * plane) = make_uint4(l[0], l[1], l[2], l[3]);
    }
  }
}

// Per field-level exponent of the largest |value| (FP16 operand scales):
// cexp[b] = max over the field-level's count doubles of floor(log2|x|),
// accumulated with atomicMax (the caller sets cexp to a very negative value
// first).  Block (x: chunk, y: field-level).
__global__ void __launch_bounds__(256) field_exponent_kernel(const double *__restrict__ src, long long count,
                                                             int *cexp) {
  pdl_wait();
  pdl_trigger();
  const int b = blockIdx.y;
  const double *p = src + (long long)b * count;
  int e = -1023;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x)
    e = max(e, f64_exponent(__ldg(p + i)));
  e = __reduce_max_sync(0xffffffffu, e);
  if ((threadIdx.x & 31) == 0) atomicMax(cexp + b, e);
}

int field_exponents(const double *src, long long count, int batch, int *cexp, cudaStream_t s) {
  if (batch <= 0) return DCCM_OK;
  if (batch > 65535) return DCCM_ERR_UNSUPPORTED;
  DCCM_CUDA(cudaMemsetAsync(cexp, 0x80, (size_t)batch * sizeof(int), s));  // 0x80808080: below any exponent
  long long bx = (count + 255) / 256;
  const long long want = (4LL * sm_count() + batch - 1) / batch;  // a few waves in all
  if (bx > want) bx = want < 1 ? 1 : want;
  DCCM_CUDA(launch_pdl(field_exponent_kernel, dim3((unsigned)bx, (unsigned)batch), dim3(256), 0, s, src, count,
                       cexp));
  return DCCM_OK;
}

int pack_spectra(Plan *const *plans, const int *batch, const double *const *spec, int ngroups, cudaStream_t s) {
  if (ngroups < 1 || ngroups > MAXG) return DCCM_ERR_UNSUPPORTED;
  PackLaunch L;
  memset(&L, 0, sizeof L);
  int ng = 0;
  long long total = 0;
  for (int g = 0; g < ngroups; ++g) {
    if (batch[g] <= 0) continue;
    const Plan &P = *plans[g];
    if (!P.d_apack || !P.d_punits) return DCCM_ERR_UNSUPPORTED;
    PackGroup &G = L.g[ng++];
    G.spec = reinterpret_cast<const double2 *>(spec[g]);
    G.units = P.d_punits;
    G.A = P.d_apack;
    G.ncoef = P.ncoef;
    G.KX = P.KX;
    G.N = P.N;
    G.C2Bp = P.C2Bp;
    G.batch = batch[g];
    G.nunits = P.npunits;
    G.nsplit = P.nsplit;
    G.cexp = P.d_cexp;
    G.t0 = total;
    total += 2LL * P.npunits * batch[g];  // a thread per (field-level, unit, parity)
    if (P.nsplit == 2) DCCM_TRY(field_exponents(spec[g], 2 * P.ncoef, batch[g], P.d_cexp, s));
  }
  L.ngroups = ng;
  L.total = total;
  if (total == 0) return DCCM_OK;
  const long long nblk = (total + 127) / 128;  // 128-thread blocks: a c3 batch (35 k units) spans every SM
  if (nblk > 0x7FFFFFFFLL) return DCCM_ERR_UNSUPPORTED;
  DCCM_CUDA(launch_pdl(pack_spectra_kernel, dim3((unsigned)nblk), dim3(128), 0, s, L));
  return DCCM_OK;
}

// ------------------------------------------------------------ tile tables
// Largest binary exponent of the table entries of each m (FP16 tables):
// dir 0 Pbar, dir 1 (w/2) Pbar, over every n >= m and latitude pair.
__global__ void table_exponent_kernel(int dir, int N, int Jh, const double *__restrict__ pnm,
                                      const double *__restrict__ w, int *emax) {
  const int m = blockIdx.y;  // block (x: entries of m, y: m)
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)(N + 1 - m) * Jh) return;
  const int jj = (int)(t % Jh);
  double x = pnm[idx_mn(N, m, m) * Jh + t];
  if (dir) x *= 0.5 * w[Jh + jj];
  atomicMax(emax + m, f64_exponent(x));
}

// FP64 split into two FP16 numbers x = hi + lo (+ dropped), once per table entry.
__device__ __forceinline__ void split2h(double x, __half &h, __half &l) {
  h = __double2half(x);
  l = __double2half(x - (double)__half2float(h));
}

// Fill the split tiles of one direction from the FP64 Pbar table: BF16 x 3,
// or FP16 hi + lo of the values times 2^eb(m).  Thread per (tile row of
// split 0, group of 8 along K).
__global__ void build_tiles_kernel(int dir, int N, int Jh, int ns, const MInfo *__restrict__ mi,
                                   const long long *__restrict__ rowstart, long long nrows0,
                                   const double *__restrict__ pnm, const double *__restrict__ w,
                                   uint16_t *__restrict__ out) {
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (tid >= nrows0 * 8) return;
  const long long r0 = tid >> 3;
  const int g8 = (int)(tid & 7);
  // find (m, p, q, r) of this split-0 row: rowstart[m] = first split-0 row index of m
  int lo = 0, hi = N + 1;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (rowstart[mid] <= r0) lo = mid;
    else hi = mid;
  }
  const int m = lo;
  const MInfo M = mi[m];
  long long rr = r0 - rowstart[m];
  const int r = (int)(rr % M.nr);
  rr /= M.nr;
  const int q = (int)(rr % M.nq);
  const int p = (int)(rr / M.nq);
  const int kv = p ? M.kv1 : M.kv0;
  const int nv = p ? M.nv1 : M.nv0;
  __align__(16) uint16_t h[8], md[8], l[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const int k = q * 64 + g8 * 8 + e;
    double x = 0.0;
    if (k < kv && r < nv) {
      if (dir == 0) {  // rows = latitude pair jj, K = n index
        const int n = m + p + 2 * k;
        x = pnm[idx_mn(N, m, n) * Jh + r];
      } else {  // rows = n index, K = latitude pair
        const int n = m + p + 2 * r;
        x = (0.5 * w[Jh + k]) * pnm[idx_mn(N, m, n) * Jh + k];
      }
    }
    if (ns == 3) {
      __nv_bfloat16 bh, bm, bl;
      split3(x, bh, bm, bl);
      h[e] = __bfloat16_as_ushort(bh);
      md[e] = __bfloat16_as_ushort(bm);
      l[e] = __bfloat16_as_ushort(bl);
    } else {
      __half hh, hl;
      split2h(ldexp(x, M.eb), hh, hl);
      h[e] = __half_as_ushort(hh);
      md[e] = __half_as_ushort(hl);
    }
  }
  const long long row_s0 = M.base + ((long long)(p * M.nq + q) * ns + 0) * M.nr + r;
  *reinterpret_cast<uint4 *>(out + row_s0 * 64 + g8 * 8) = *reinterpret_cast<const uint4 *>(h);
  *reinterpret_cast<uint4 *>(out + (row_s0 + M.nr) * 64 + g8 * 8) = *reinterpret_cast<const uint4 *>(md);
  if (ns == 3)
    *reinterpret_cast<uint4 *>(out + (row_s0 + 2LL * M.nr) * 64 + g8 * 8) = *reinterpret_cast<const uint4 *>(l);
}

// Host metadata for one direction's table.
struct TabMeta {
  std::vector<MInfo> mi;
  std::vector<long long> rowstart;  // split-0 rows before m
  std::vector<int4> items;          // (m, 0, nt, 0) of one 128-column block
  long long rows = 0, rows0 = 0;
};

static TabMeta make_meta(int dir, const Plan &P, const std::vector<int> &emax, int tn) {
  const int N = P.N, Jh = P.Jh;
  TabMeta t;
  t.mi.resize(N + 1);
  t.rowstart.resize(N + 2);
  long long base = 0, r0 = 0;
  for (int m = 0; m <= N; ++m) {
    MInfo &M = t.mi[m];
    const int c0 = count_np(N, m, 0), c1 = count_np(N, m, 1);
    if (dir == 0) {
      M.kv0 = c0; M.kv1 = c1;
      M.nv0 = Jh; M.nv1 = Jh;
      M.nr = (Jh + 15) / 16 * 16;
      M.nq = (c0 + 63) / 64;
      M.x0 = P.xoff[2 * m];
      M.x1 = P.xoff[2 * m + 1];
    } else {
      M.kv0 = Jh; M.kv1 = Jh;
      M.nv0 = c0; M.nv1 = c1;
      M.nr = (c0 + 15) / 16 * 16;
      M.nq = (Jh + 63) / 64;
      M.x0 = 2 * m * Jh;
      M.x1 = (2 * m + 1) * Jh;
    }
    M.base = base;
    M.eb = P.nsplit == 2 ? 14 - emax[m] : 0;
    t.rowstart[m] = r0;
    base += 2LL * M.nq * P.nsplit * M.nr;
    r0 += 2LL * M.nq * M.nr;
    for (int nt = 0; nt < (M.nr + tn - 1) / tn; ++nt) t.items.push_back(make_int4(m, 0, nt, 0));
  }
  t.rowstart[N + 1] = r0;
  t.rows = base;
  t.rows0 = r0;
  return t;
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *,
                                  CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                  CUtensorMapFloatOOBfill);

static EncodeTiledFn get_encode() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

// bf16 (or fp16) tensor map with a 128-byte swizzle; dims/strides/box
// innermost first.
static int encode_bf16(CUtensorMap *map, void *base, int rank, const cuuint64_t *dims, const cuuint64_t *strides,
                       const cuuint32_t *box, bool fp16 = false) {
  EncodeTiledFn enc = get_encode();
  if (!enc) return DCCM_ERR_UNSUPPORTED;
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = enc(map, fp16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16,
                         (cuuint32_t)rank, base, dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? DCCM_OK : DCCM_ERR_UNSUPPORTED;
}

static int build_one(Plan &P, int dir, TileTable &T) {
  std::vector<int> emax(P.N + 1, 0);
  if (P.nsplit == 2) {  // per-m scale exponents of the FP16 tables
    int *de;
    DCCM_CUDA(cudaMalloc(&de, (P.N + 1) * sizeof(int)));
    DCCM_CUDA(cudaMemset(de, 0x80, (P.N + 1) * sizeof(int)));
    const long long nt = (long long)(P.N + 1) * P.Jh;
    table_exponent_kernel<<<dim3((unsigned)((nt + 255) / 256), (unsigned)(P.N + 1)), 256>>>(dir, P.N, P.Jh,
                                                                                        P.d_pnm, P.d_w, de);
    DCCM_LAUNCH_CHECK();
    DCCM_CUDA(cudaMemcpy(emax.data(), de, (P.N + 1) * sizeof(int), cudaMemcpyDeviceToHost));
    cudaFree(de);
    for (int &e : emax) e = e < -1000 ? -1000 : e;  // an all-zero m: any scale
  }
  // N rows of a tile (B box rows, TMEM columns of an accumulator): 64 where
  // every tile fits, and always for the analysis, whose epilogue (through
  // shared memory) then overlaps the next item's MMAs in the second
  // accumulator set (T341 x 192 field-levels: 184 -> 162 us); the
  // synthesis keeps 128-row tiles for larger tables (with 64 it reloads
  // each spectra tile twice as often: 194 -> 214 us).
  int nrmax = 16;
  for (int m = 0; m <= P.N; ++m) {
    const int nr = dir == 0 ? (P.Jh + 15) / 16 * 16 : (count_np(P.N, m, 0) + 15) / 16 * 16;
    nrmax = nr > nrmax ? nr : nrmax;
  }
  const int tn = (nrmax <= 64 || dir == 1) ? 64 : 128;
  TabMeta meta = make_meta(dir, P, emax, tn);
  T.rows = meta.rows;
  T.base.assign(P.N + 1, 0);
  for (int m = 0; m <= P.N; ++m) T.base[m] = meta.mi[m].base;
  DCCM_CUDA(cudaMalloc(&T.d, (size_t)meta.rows * 64 * sizeof(uint16_t)));
  MInfo *dmi;
  long long *drs;
  DCCM_CUDA(cudaMalloc(&dmi, meta.mi.size() * sizeof(MInfo)));
  T.d_mi = dmi;
  DCCM_CUDA(cudaMalloc(&drs, meta.rowstart.size() * sizeof(long long)));
  DCCM_CUDA(cudaMemcpy(dmi, meta.mi.data(), meta.mi.size() * sizeof(MInfo), cudaMemcpyHostToDevice));
  DCCM_CUDA(cudaMemcpy(drs, meta.rowstart.data(), meta.rowstart.size() * sizeof(long long),
                       cudaMemcpyHostToDevice));
  // Work items (m, -, nt) of one 128-column block, heavy (small m) first;
  // a launch runs each of them for every column block of its batch.
  const std::vector<int4> &items = meta.items;
  DCCM_CUDA(cudaMalloc(&T.d_items, items.size() * sizeof(int4)));
  DCCM_CUDA(cudaMemcpy(T.d_items, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice));
  const long long nthr = meta.rows0 * 8;
  if (nthr > 0) {
    build_tiles_kernel<<<(unsigned)((nthr + 255) / 256), 256>>>(dir, P.N, P.Jh, P.nsplit, dmi, drs, meta.rows0,
                                                               P.d_pnm, P.d_w, T.d);
    DCCM_LAUNCH_CHECK();
  }
  DCCM_CUDA(cudaDeviceSynchronize());
  cudaFree(drs);
  T.ntmax = tn;
  {  // B boxes of ntmax rows
    const cuuint64_t dims[2] = {64, (cuuint64_t)meta.rows};
    const cuuint64_t str[1] = {128};
    const cuuint32_t box[2] = {64, (cuuint32_t)T.ntmax};
    DCCM_TRY(encode_bf16(&T.map, T.d, 2, dims, str, box, P.nsplit == 2));
  }
  const cuuint64_t ns = (cuuint64_t)P.nsplit;
  if (dir == 0) {  // Apack[ns][C2Bp][KX], box 64 (K) x 128 (c)
    const cuuint64_t dims[3] = {(cuuint64_t)P.KX, (cuuint64_t)P.C2Bp, ns};
    const cuuint64_t str[2] = {(cuuint64_t)P.KX * 2, (cuuint64_t)P.KX * 2 * P.C2Bp};
    const cuuint32_t box[3] = {64, 128, 1};
    DCCM_TRY(encode_bf16(&T.amap, P.d_apack, 3, dims, str, box, P.nsplit == 2));
  } else {  // G3[ns][(N+1) 2 Jh][C2Bp], box 64 (c) x 64 (K)
    const cuuint64_t rows = (cuuint64_t)(P.N + 1) * 2 * P.Jh;
    const cuuint64_t dims[3] = {(cuuint64_t)P.C2Bp, rows, ns};
    const cuuint64_t str[2] = {(cuuint64_t)P.C2Bp * 2, (cuuint64_t)P.C2Bp * 2 * rows};
    const cuuint32_t box[3] = {64, 64, 1};
    DCCM_TRY(encode_bf16(&T.amap, P.d_work, 3, dims, str, box, P.nsplit == 2));
  }
  T.map_ok = true;
  T.items_per_ct = (int)meta.items.size();
  return DCCM_OK;
}

// Apack layout (segments of (m, p) along x, each rounded up to 16) and the
// column of every coefficient; the buffer is zeroed once so the segment
// padding contributes nothing.
static int build_pack(Plan &P) {
  P.C2Bp = (2 * P.max_batch + 7) / 8 * 8;
  P.xoff.assign(2 * (P.N + 1), 0);
  long long x = 0;
  for (int m = 0; m <= P.N; ++m)
    for (int p = 0; p < 2; ++p) {
      P.xoff[2 * m + p] = (int)x;
      x += (count_np(P.N, m, p) + 15) / 16 * 16;
    }
  P.KX = x;
  if (P.KX >= (1LL << 31)) return DCCM_ERR_UNSUPPORTED;
  // pack units (m, q): coefficients n = m + 16 q .. + 15, columns 8 q .. 8 q + 7
  // of both parity segments (the kernel skips a parity's run that starts at
  // or past that parity's coefficient count)
  std::vector<int4> units;
  for (int m = 0; m <= P.N; ++m)
    for (int q = 0; m + 16 * q <= P.N; ++q)
      units.push_back(make_int4(m, q, P.xoff[2 * m] + 8 * q, P.xoff[2 * m + 1] + 8 * q));
  P.npunits = (int)units.size();
  DCCM_CUDA(cudaMalloc(&P.d_punits, units.size() * sizeof(int4)));
  DCCM_CUDA(cudaMemcpy(P.d_punits, units.data(), units.size() * sizeof(int4), cudaMemcpyHostToDevice));
  const size_t bytes = (size_t)P.nsplit * P.C2Bp * P.KX * sizeof(uint16_t);
  DCCM_CUDA(cudaMalloc(&P.d_apack, bytes));
  DCCM_CUDA(cudaMemset(P.d_apack, 0, bytes));
  return DCCM_OK;
}

// Called after d_work exists (the forward A map points into it).
int build_tiles(Plan &P) {
  DCCM_TRY(build_pack(P));
  DCCM_TRY(build_one(P, 0, P.tinv));
  DCCM_TRY(build_one(P, 1, P.tfwd));
  return DCCM_OK;
}

template <bool NARROW> static size_t tc_smem_bytes() {
  return 1024 + (size_t)TcShape<NARROW>::NSTAGE * TcShape<NARROW>::STAGE_BYTES + 128 + EP_BYTES;
}

// One persistent launch over ngroups plans (truncation groups) of one
// direction: dir 0 (inverse) reads the plan's packed spectra (pack_spectra
// must have run on the same stream) and writes out[g] = F (float); dir 1
// reads the plan's G3 (written by the forward FFT) and writes out[g] =
// spectra (double).  in[] is unused (the operands come by TMA).
int legendre_tc_multi(Plan *const *plans, const int *batch, const void *const *in, void *const *out,
                      int ngroups, int dir, cudaStream_t s) {
  (void)in;
  static bool attr_done = false;
  if (ngroups < 1 || ngroups > MAXG) return DCCM_ERR_UNSUPPORTED;
  if (!attr_done) {
    DCCM_CUDA(cudaFuncSetAttribute(legendre_tc_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)tc_smem_bytes<false>()));
    DCCM_CUDA(cudaFuncSetAttribute(legendre_tc_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)tc_smem_bytes<true>()));
    DCCM_CUDA(cudaFuncSetAttribute(legendre_tc_kernel<true>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                   (int)cudaSharedmemCarveoutMaxShared));
    attr_done = true;
  }
  TcLaunch L;
  memset(&L, 0, sizeof L);
  int ntmax = 64, ng = 0, items = 0;
  for (int g = 0; g < ngroups; ++g) {
    const TileTable &T = dir == 0 ? plans[g]->tinv : plans[g]->tfwd;
    if (!T.map_ok) return DCCM_ERR_UNSUPPORTED;
    ntmax = T.ntmax > ntmax ? T.ntmax : ntmax;
  }
  const bool narrow = ntmax <= 64 && tunables().tc_shape == 1;
  for (int g = 0; g < ngroups; ++g) {
    if (batch[g] <= 0) continue;
    Plan &P = *plans[g];
    const TileTable &T = dir == 0 ? P.tinv : P.tfwd;
    TcArgs &a = L.g[ng];
    a.dir = dir;
    a.batch = batch[g];
    a.N = P.N;
    a.Jh = P.Jh;
    a.ncoef = P.ncoef;
    a.mi = (const MInfo *)T.d_mi;
    a.items = T.d_items;
    a.err = plans[0]->d_err;
    a.ntmax = ntmax;
    a.brows = T.ntmax;
    a.nacc = 8 * ntmax <= (narrow ? TcShape<true>::TMEM_COLS : TcShape<false>::TMEM_COLS) ? 2 : 1;
    a.nsplit = P.nsplit;
    a.cexp = dir == 0 ? P.d_cexp : P.d_cexp + P.max_batch;
    if (dir == 0) a.F = (float *)out[g];
    else a.spec_out = (double *)out[g];
    L.map[ng] = T.map;
    L.amap[ng] = T.amap;
    L.start[ng] = items;
    a.nct = (2 * a.batch + 127) / 128;
    items += a.nct * T.items_per_ct;
    ++ng;
  }
  L.start[ng] = items;
  L.ngroups = ng;
  L.wait_ns = tunables().wait_limit_ms > 0 ? 1000000ull * (unsigned long long)tunables().wait_limit_ms
                                           : WAIT_LIMIT_NS;
  L.withhold = tunables().tc_withhold_loads;
  if (items <= 0) return DCCM_OK;
  const int resident = (narrow ? TcShape<true>::MIN_CTAS : 1) * sm_count();  // persistent: at most one wave
  int ctas = tunables().tc_ctas > 0 ? tunables().tc_ctas : resident;
  ctas = ctas < resident ? ctas : resident;
  const int grid = items < ctas ? items : ctas;
  if (narrow)
    DCCM_CUDA(launch_pdl(legendre_tc_kernel<true>, dim3(grid), dim3(tc_threads<true>()), tc_smem_bytes<true>(), s, L));
  else
    DCCM_CUDA(launch_pdl(legendre_tc_kernel<false>, dim3(grid), dim3(tc_threads<false>()), tc_smem_bytes<false>(), s, L));
  return DCCM_OK;
}

int legendre_inv_tc(Plan &P, int batch, const double *spec, float *F, cudaStream_t s) {
  if (batch <= 0) return DCCM_OK;
  Plan *pp = &P;
  DCCM_TRY(pack_spectra(&pp, &batch, &spec, 1, s));
  const void *in = spec;
  void *out = F;
  return legendre_tc_multi(&pp, &batch, &in, &out, 1, 0, s);
}

int legendre_fwd_tc(Plan &P, int batch, const void *G3, double *spec, cudaStream_t s) {
  if (batch <= 0) return DCCM_OK;
  Plan *pp = &P;
  const void *in = G3;
  void *out = spec;
  return legendre_tc_multi(&pp, &batch, &in, &out, 1, 1, s);
}

}  // namespace sht
}  // namespace dccm
