// Tiled fused push + deposit: one CTA per tile of cells.
//
// The species' particles are stored tile-major (PIC_SORT_TILED), so the
// particles of a tile are one contiguous range per species and are read and
// written back fully coalesced. The CTA
//   1. stages the E/B window of its tile (tile + interpolation halo + a drift
//      margin of M cells) in shared memory: one TMA box load (all six
//      components) that runs while the CTA clears its J window and scans its
//      particles' weights, or a strided copy loop for a window that wraps
//      across a periodic edge;
//   2. pushes every particle of the tile (all species) gathering E/B from
//      shared memory and depositing its current into a shared-memory J window
//      (tile + deposit halo + margin); in FP32 a particle whose shape
//      support moved is deposited after the pushes, from a record (DepStage),
//   3. adds the J window to global J once, wrapping periodic images onto
//      their active cells (the fold SynchronizeFields performs in the
//      reference, src/framework/domain/metadomain_comm.cpp:408-562).
//
// Accumulation in the J window: fixed point split over 32-bit words.
// 32-bit integer shared-memory atomics are the fastest this GPU has (a
// microbenchmark measured 9.1 Top/s, against 2.8 for float, 1.6 for 64-bit
// integers and 0.5 for double), and integer sums do not depend on the order
// of the additions. Each tile scales contributions by a power of two 2^s so
// that |v 2^s| < 2^b, rounds them to integers (exact up to the quantisation
// 2^-s) and adds them as 32-bit words: X modulo 2^32 and X >> 12 (float),
// or three 16-bit words and a signed top word (double). With N
// particles in the tile no cell takes more than N additions per component,
// so b = min(30, 43 - log2 N) (float; 29 bits at 16k particles) or
// b = 62 - log2 N (double) overflows neither a word nor the 64-bit total.
// The tile's sum is exact and
// independent of the order of the additions; each cell is rounded to real
// once, at the flush. A tile denser than the words allow (N > 2^20 in float,
// 2^16 in double) accumulates in real_t atomics instead.
//
// A particle that has drifted more than M cells outside its tile since the
// last tiled sort, or whose stencil can reach the ghost layers of a
// non-periodic axis, is not touched here: it is appended to the species'
// overflow list and pushed afterwards by the per-particle kernel (global
// gathers, global atomics, the reference's coordinates). Results therefore
// never depend on the sort interval, and the hot kernel holds only the
// shared-memory path. Arithmetic per particle is the same code as the
// untiled kernel.
#pragma once

#include <type_traits>

#include "push_deposit.cuh"
#include "tma.cuh"

namespace pic {

constexpr int kMaxTiledSpecies = 4;
constexpr int kDriftMargin     = 1;

// the J-window accumulator words of one precision (see the header)
template <typename real>
struct FixedAcc;
template <>
struct FixedAcc<float> {
  static constexpr int     WORDS = 2;
  static constexpr int64_t NMAX  = (1 << 20) - 1;  // low-word sums stay below 2^32
  // b = 43 - log2 N keeps the high-word sums below 2^31; capped at 30 so that
  // the scaled contribution converts to a 32-bit integer
  __device__ static int bits(int64_t n) { return min(30, 43 - (n > 1 ? 64 - __clzll(n - 1) : 0)); }
  // v arrives already scaled by 2^s (|v| < 2^b). X = round(v) goes into two
  // words with integer adds: the low word sums X itself modulo 2^32, the
  // high word sums the floored quotient hi = X >> 12. Over the N additions
  // sum X = 4096 H + r with H the high word's total and r = sum (X mod 4096)
  // in [0, 4096 N), below 2^32 for N <= NMAX; the low word fixes r modulo
  // 2^32, so r = L - 4096 H (mod 2^32). Both sums are exact and independent
  // of the order of the additions, and the low word needs no mask.
  __device__ static void add(unsigned* w, int plane, float v) {
    const int X = __float2int_rn(v);
    atomicAdd(w, (unsigned)X);
    atomicAdd(w + plane, (unsigned)(X >> 12));
  }
  __device__ static bool nonzero(const unsigned* w, int plane) { return (w[0] | w[plane]) != 0u; }
  __device__ static long long total(const unsigned* w, int plane) {
    const unsigned H = w[plane];
    return (long long)(int)H * 4096 + (long long)(w[0] - (H << 12));
  }
  __device__ static float to_real(long long t, float unscale) { return __ll2float_rn(t) * unscale; }
};
template <>
struct FixedAcc<double> {
  static constexpr int     WORDS = 4;
  static constexpr int64_t NMAX  = 1 << 16;  // 16-bit word sums stay below 2^32
  // the 64-bit total of N additions must not overflow either
  __device__ static int bits(int64_t n) { return 62 - (n > 1 ? 64 - __clzll(n - 1) : 0); }
  __device__ static void add(unsigned* w, int plane, double v) {
    const long long X = __double2ll_rn(v);  // v arrives scaled by 2^s
    atomicAdd(w, (unsigned)(X & 0xFFFF));
    atomicAdd(w + plane, (unsigned)((X >> 16) & 0xFFFF));
    atomicAdd(w + 2 * plane, (unsigned)((X >> 32) & 0xFFFF));
    atomicAdd(w + 3 * plane, (unsigned)(int)(X >> 48));
  }
  __device__ static bool nonzero(const unsigned* w, int plane) {
    return (w[0] | w[plane] | w[2 * plane] | w[3 * plane]) != 0u;
  }
  __device__ static long long total(const unsigned* w, int plane) {
    const unsigned long long t = ((unsigned long long)(long long)(int)w[3 * plane] << 48) +
                                 ((unsigned long long)w[2 * plane] << 32) +
                                 ((unsigned long long)w[plane] << 16) + w[0];
    return (long long)t;
  }
  __device__ static double to_real(long long t, double unscale) {
    return __ll2double_rn(t) * unscale;
  }
};

// tile shape per (dimension, precision, order): the shared-memory windows
// must fit one CTA's 227 KB
template <int D, typename real, int O>
struct TileShape {
  // 2D: 16 x 8 cells. The 512^2 pair plasma (2 x 16 ppc) ran push+deposit in
  // 0.578 ms with 32 x 32 tiles (256 CTAs, 0.56 waves), 0.456 ms with
  // 16 x 16, 0.419 ms with 16 x 8 and 0.429 ms with 8 x 8.
  // NT threads per CTA; MINB CTAs per SM asked of the register allocator.
  // The kernel is latency-bound, so warps per SM pay: FP32 at 256 threads ran
  // 0.543 ms with the allocator's 80 registers (3 CTAs/SM), 0.388 ms at 64
  // (4 CTAs), 0.350 ms at 48 (5 CTAs, no spill) and 0.366 ms at 40 (6 CTAs,
  // spilling); 512 threads x 2 gave 0.408 ms
  static constexpr int X = 16, Y = 8, Z = 1, NT = 256,
                       MINB = sizeof(real) == 4 ? (O == 3 ? 4 : 5) : 1;  // order 3 spills at 5
};
// 3D FP32 at order 3: 8^3 cells, so that two copies of the J window fit
// (measured on the 96^3 sweep plasma, 2 x 32 ppc: 28.1 ms per step against
// 34.7 ms with one copy and 16 x 8 x 4 tiles). At order 2 the copies did not
// pay (50.5 against 48.1 ms on the 256^3 turbulence plasma, 2 x 8 ppc; with
// the deposit records and the even-odd rows 34.5 against 28.8 ms): its warps
// span several cells, so fewer lanes share a word.
// Threads per CTA: one CTA per SM (the shared memory), so the thread count
// sets the warps that hide the kernel's latencies, and the register file
// sets what each may use. Push+deposit of the 256^3 turbulence plasma
// (order 2) took 44.96 ms at 512 threads (128 registers), 40.26 at 640 (96),
// 38.38 at 768 (80), 38.19 at 896 (72) and 36.31 at 1024 (64, no spill); the
// 96^3 sweep plasma (order 3) 27.00, 25.55, 25.62, 26.30 and 26.86 ms (at
// 1024 its registers spill)
template <int O>
struct TileShape<3, float, O> {
  static constexpr int X = (O == 3 ? 8 : 16), Y = 8, Z = 8, NT = (O == 3 ? 640 : 1024), MINB = 1;
};
// FP64 (8 x 8 x 4 cells): 256, 384, 512 and 768 threads ran the FP64 twin of
// the sweep plasma (order 3) at 150, 151, 145 and 137 M particle-steps/s
template <int O>
struct TileShape<3, double, O> {
  static constexpr int X = 8, Y = 8, Z = 4, NT = 384, MINB = 1;
};

// window halos (cells below / above the tile) of the interpolation and the
// deposit stencils at order O, plus the drift margin
template <int O>
struct Halo {
  static constexpr int E_LO = (O == 3 ? 2 : 1) + kDriftMargin;
  static constexpr int E_HI = (O >= 2 ? 2 : 1) + kDriftMargin;
  static constexpr int J_LO = (O >= 2 ? 2 : 1) + kDriftMargin;
  static constexpr int J_HI = (O >= 2 ? 3 : 2) + kDriftMargin;
};

template <typename real>
struct TiledSpecies {
  SpeciesPtrs    sp;
  const int32_t* tile_start;  // ntiles + 1 offsets into the particle arrays
  real           ndth, charge;
  int            vay;
  int32_t*       ovf;         // particles left to the per-particle kernel
  unsigned*      ovf_count;
};

// Deposit records (FP32: 3D orders 1-3, 2D orders 1-2; 2D records carry the
// out-of-plane velocity in place of the third offsets). Most particles end a
// step with both shape supports starting at the same node on every axis
// (support_unmoved): their Esirkepov box is (O + 1) wide on each axis, a
// stencil the compiler unrolls to its exact extent (54 of the 144 entries at
// order 2). A warp deposits those at once. The others, whose box is O + 2
// wide on some axis, are appended as 32-byte records to a buffer in global
// memory (L2-resident: a few hundred KB per CTA, written and read back by
// the same CTA) and deposited after the tile's pushes by full warps. So no
// warp runs the wide stencil for one lane, and J is unchanged to the bit:
// the window's integer sums do not depend on the order of the additions.
// A CTA claims one of nslots buffers (nslots >= the CTAs that can be
// resident at once); without one, or past cap records, it deposits at once.
struct DepStage {
  uint4*    rec    = nullptr;  // nslots * cap records of two uint4
  unsigned* claim  = nullptr;  // nslots words: 0 free, 1 held
  int       nslots = 0, cap = 0;
};
// records per 3D buffer (256 KB); twice that at order 3, a quarter in 2D
constexpr int kStageCap = 8192;

// drops the 128-byte line at p (128-byte aligned) from L2 without writing it
// back; its contents are undefined until written again
__device__ __forceinline__ void discard_l2_line(const void* p) {
  asm volatile("discard.global.L2 [%0], 128;" ::"l"(p) : "memory");
}

template <typename real>
struct TiledArgs {
  TiledSpecies<real> s[kMaxTiledSpecies];
  int                nsp;
  PushConsts         pc;
  int                periodic[3];
  int                ntiles[3];
  int                tile0, tile1;  // linear tiles [tile0, tile1) of this launch
  FieldView<real>    EB;
  FieldView<real>    J;
  real               dt, dx, inv_dt;
  int                write_prev;
  unsigned long long* err;
  // tiled tensor map of EB (x, y, [z], component) with the E-window box;
  // eb_tma = 0 when the field array does not meet TMA's alignment rules
  alignas(64) CUtensorMap eb_map;
  int                eb_tma;
  // FP32: the exact 64-bit accumulator the tile sums are flushed into (null:
  // float atomics into J)
  FixedJ             fj;
  // 3D FP32: where a tile's moved-support particles wait for their deposit
  DepStage           st;
  // warps taken lane_stride at a time read their particles interleaved
  // (1, 2 or 4; a divisor of the CTA's warps). A warp of a cell-sorted tile
  // then spans 32 lane_stride / ppc cells; about four measured best: on
  // the 256^3 turbulence plasma (8 ppc per species) strides 1, 2 and 4 took
  // 28.9, 29.6 and 30.4 ms of push+deposit, on the 96^3 sweep plasma (32)
  // 24.1, 21.2 and 20.4 ms, on the 512^2 pair plasma (16) 0.333, 0.323 and
  // 0.330 ms
  int                lane_stride = 1;
};

template <int D, int O, typename real>
struct TiledGeom {
  using TS                = TileShape<D, real, O>;
  static constexpr int TX = TS::X, TY = TS::Y, TZ = (D == 3 ? TS::Z : 1);
  static constexpr int NT = TS::NT;
  using H                 = Halo<O>;
  static constexpr int WE0 = TX + H::E_LO + H::E_HI;
  static constexpr int WE1 = TY + H::E_LO + H::E_HI;
  static constexpr int WE2 = D == 3 ? TZ + H::E_LO + H::E_HI : 1;
  static constexpr int WJ0 = TX + H::J_LO + H::J_HI;
  static constexpr int WJ1 = TY + H::J_LO + H::J_HI;
  static constexpr int WJ2 = D == 3 ? TZ + H::J_LO + H::J_HI : 1;
  static constexpr int NJ  = WJ0 * WJ1 * WJ2;
  // J window: FixedAcc<real>::WORDS planes of 3 * NJ 32-bit words, in COPIES
  // copies (3D FP32 at order 3: two, one per lane parity) COPY words apart.
  // Two copies in 2D FP32 did not pay: the 512^2 pair plasma's push+deposit
  // took 0.325 ms against 0.322 ms with one
  static constexpr int    WORDS      = FixedAcc<real>::WORDS;
  static constexpr int    PLANE      = 3 * NJ;
  static constexpr int    COPIES     = (D == 3 && sizeof(real) == 4 && O == 3) ? 2 : 1;
  // moved-support particles deposited from records (DepStage), orders 1-3.
  // At order 3 the buffers hold twice the records: the sweep plasma
  // (theta = 1, 8^3-cell tiles of 2 x 32 ppc) moves 40 % of its supports;
  // with 8192 records per buffer its push+deposit on 96^3 went from 25.0 to
  // 27.5 ms, with 16384 (and the lane stride) from 20.5 to 19.6 ms
  // 2D at order 3 would spill at its four CTAs per SM, so it deposits at once
  static constexpr bool   STAGE      = sizeof(real) == 4 && O >= 1 && (D == 3 || O <= 2);
  // the copies start 16 banks apart: one word in both copies falls in
  // two different banks
  static constexpr int    COPY       = WORDS * PLANE + ((16 - (WORDS * PLANE) % 32) + 32) % 32;
  static constexpr size_t jw_bytes   = 4 * (size_t)(COPIES == 1 ? WORDS * PLANE : COPIES * COPY);
  // E window rows: a TMA box row is a multiple of 16 bytes and starts on a
  // 16-byte boundary, so the row is widened to WEX elements and the window
  // sits R = (x start mod A) elements into it (A elements per 16 bytes)
  static constexpr int    A          = 16 / (int)sizeof(real);
  static constexpr int    WEX_TMA    = ((WE0 + A - 1 + A - 1) / A) * A;
  static constexpr size_t kSmemMax   = 232448 - 128;  // per-CTA limit less the static words
  static constexpr bool fits(int wx, int wy) {
    return ((sizeof(real) * 6 * (size_t)wx * wy * WE2 + 127) / 128) * 128 + jw_bytes <= kSmemMax;
  }
  // The interpolation's lanes in one cell read x, x + 1, the next row and the
  // next plane of a window row: the row and plane strides must differ in
  // shared-memory bank (mod 32 words) or those reads conflict. The box's y
  // extent is padded (rows beyond the window are loaded and never read)
  // until x, x + 1, + row, + plane and their sums fall in 8 distinct banks.
  static constexpr bool banks_distinct(int wx, int wy) {
    // word offsets of the eight reads; a read of real_t covers w words
    const int w = (int)sizeof(real) / 4, row = wx * w, pl = wx * wy * w;
    const int o[8] = { 0, w, row, row + w, pl, pl + w, row + pl, row + pl + w };
    for (int i = 0; i < 8; ++i)
      for (int j = i + 1; j < 8; ++j) {
        const int d = ((o[i] - o[j]) % 32 + 32) % 32;
        if (d < w || d > 32 - w) return false;
      }
    return true;
  }
  static constexpr int pick_wey() {
    int best = WE1;
    for (int y = WE1 + 3; y >= WE1; --y)
      if (D == 3 && banks_distinct(WEX_TMA, y) && fits(WEX_TMA, y)) best = y;
    return best;
  }
  static constexpr bool   TMA        = fits(WEX_TMA, WE1);
  static constexpr int    WEX        = TMA ? WEX_TMA : WE0;
  static constexpr int    WEY        = TMA ? pick_wey() : WE1;
  static constexpr int    NE         = WEX * WEY * WE2;
  static constexpr size_t eb_bytes   = sizeof(real) * 6 * (size_t)NE;
  static constexpr size_t smem_bytes = ((eb_bytes + 127) / 128) * 128 + jw_bytes;
};

// wraps a ghost-free coordinate of a periodic axis into [0, n)
__device__ __forceinline__ int wrap_periodic(int x, int n) {
  x %= n;
  return x < 0 ? x + n : x;
}

template <int D, int O, typename real>
__global__ void __launch_bounds__(TileShape<D, real, O>::NT, TileShape<D, real, O>::MINB)
    k_push_deposit_tiled(const __grid_constant__ TiledArgs<real> a) {
  using G               = TiledGeom<D, O, real>;
  using H               = Halo<O>;
  using FA              = FixedAcc<real>;
  constexpr int  NT     = G::NT;
  constexpr int  M      = kDriftMargin;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  real*          EBs = reinterpret_cast<real*>(smem_raw);
  unsigned*      Jw  = reinterpret_cast<unsigned*>(smem_raw + ((G::eb_bytes + 127) / 128) * 128);
  real*          Jr  = reinterpret_cast<real*>(Jw);  // real_t accumulation of dense tiles
  __shared__ unsigned int s_qmax;  // bit pattern of the tile's largest |q w| max(1/dt, 1)
  __shared__ __align__(8) unsigned long long s_bar;  // completion of the E-window load
  __shared__ int      s_slot;  // the claimed record buffer, -1 for none
  __shared__ unsigned s_nrec;  // records appended so far

  const int t  = blockIdx.x + a.tile0;
  const int tx = t % a.ntiles[0];
  const int ty = (t / a.ntiles[0]) % a.ntiles[1];
  const int tz = D == 3 ? t / (a.ntiles[0] * a.ntiles[1]) : 0;
  const int T0[3] = { tx * G::TX, ty * G::TY, tz * G::TZ };
  const int ng    = a.pc.ng;

  // 1. E/B window, ghost-inclusive start g0 along each axis; the window's
  //    rows start R elements into the widened shared rows
  const int g0[3] = { ng + T0[0] - H::E_LO, ng + T0[1] - H::E_LO,
                      D == 3 ? ng + T0[2] - H::E_LO : 0 };
  const int R     = G::TMA ? (g0[0] & (G::A - 1)) : 0;
  bool      tma   = false;
  if constexpr (G::TMA) {
    // one box load covers the window when no periodic axis wraps inside it
    // (beyond a non-periodic edge the load's zero fill is what the copy
    // loop writes too)
    const int we[3] = { G::WE0, G::WE1, G::WE2 };
    tma = a.eb_tma != 0 && (smem_addr(EBs) & 127u) == 0u;
#pragma unroll
    for (int d = 0; d < D; ++d)
      if (a.periodic[d] && (g0[d] < 0 || g0[d] + we[d] > a.pc.ext[d])) tma = false;
  }
  const unsigned bar = smem_addr(&s_bar);
  if (tma) {
    if (threadIdx.x == 0) {
      mbar_init(bar, 1);
      mbar_expect_tx(bar, (unsigned)G::eb_bytes);
      if constexpr (D == 3) tma_load_4d(smem_addr(EBs), &a.eb_map, bar, g0[0] - R, g0[1], g0[2], 0);
      else                  tma_load_3d(smem_addr(EBs), &a.eb_map, bar, g0[0] - R, g0[1], 0);
    }
  } else {
    // reads ghost cells where the window overlaps them and the periodic
    // image beyond (zero beyond a non-periodic edge: no valid particle's
    // stencil reaches there)
    for (int idx = threadIdx.x; idx < 6 * G::WE0 * G::WE1 * G::WE2; idx += NT) {
      int       r  = idx;
      const int wi = r % G::WE0;
      r /= G::WE0;
      const int wj = r % G::WE1;
      r /= G::WE1;
      const int wk = r % G::WE2;
      const int c  = r / G::WE2;
      int       gc[3] = { T0[0] - H::E_LO + wi, T0[1] - H::E_LO + wj,
                          D == 3 ? T0[2] - H::E_LO + wk : 0 };
      bool      inside = true;
#pragma unroll
      for (int d = 0; d < D; ++d) {
        if (gc[d] < -ng || gc[d] >= a.pc.n[d] + ng) {
          if (a.periodic[d]) gc[d] = wrap_periodic(gc[d], a.pc.n[d]);
          else inside = false;
        }
      }
      EBs[R + wi + G::WEX * (wj + G::WEY * (wk + G::WE2 * c))] =
          inside ? a.EB.ld(gc[0] + ng, gc[1] + ng, D == 3 ? gc[2] + ng : 0, c) : (real)0;
    }
  }
  for (int idx = threadIdx.x; idx < (G::COPIES == 1 ? G::WORDS * G::PLANE : G::COPIES * G::COPY);
       idx += NT)
    Jw[idx] = 0u;
  // largest contribution bound of the tile, |q w| max(1/dt, 1), and its
  // particle count (an upper bound on the additions any cell receives)
  if (threadIdx.x == 0) {
    s_qmax = 0u;
    s_nrec = 0u;
    s_slot = -1;
    if (G::STAGE && a.st.rec) {
      // one attempt per buffer, starting where this CTA's predecessors by
      // index left theirs: no wait
      for (int k = 0; k < a.st.nslots; ++k) {
        const int sl = (int)((blockIdx.x + (unsigned)k) % (unsigned)a.st.nslots);
        if (atomicCAS(a.st.claim + sl, 0u, 1u) == 0u) {
          s_slot = sl;
          break;
        }
      }
    }
  }
  __syncthreads();
  // (with the exact global accumulator the bound is the call's, known already)
  const bool global_unit = sizeof(real) == 4 && a.fj.p != nullptr;
  float      qmax = 0.f;
  int64_t    ntile = 0;
  for (int s = 0; s < a.nsp; ++s) {
    const real*   w  = (const real*)a.s[s].sp.w;
    const float   qs = fabsf((float)a.s[s].charge);
    const int64_t lo = a.s[s].tile_start[t], hi = a.s[s].tile_start[t + 1];
    ntile += hi - lo;
    if (global_unit) continue;
    for (int64_t p = lo + threadIdx.x; p < hi; p += NT) qmax = fmaxf(qmax, fabsf((float)w[p]) * qs);
  }
  qmax *= fmaxf((float)a.inv_dt, 1.f);
  atomicMax(&s_qmax, __float_as_uint(qmax));  // non-negative floats order as their bits
  __syncthreads();
  const bool fixed = ntile <= FA::NMAX;
  real       scale = 1, unscale = 1;
  int        ex = 0, b = FA::bits(ntile);
  if (global_unit) {
    // the call's bound, and no more bits than the global unit has, so that
    // a tile total becomes global units by a left shift
    ex = a.fj.exponent();
    b  = min(b, a.fj.bits);
  } else {
    frexpf(__uint_as_float(s_qmax) * 1.0000002f, &ex);  // |contribution| < 2^ex
  }
  scale   = (real)ldexp(1.0, b - ex);
  unscale = (real)ldexp(1.0, ex - b);

  if (tma) {
    // every thread waits for the window; a lost wait (the limit ran out on
    // any thread) abandons the tile on all of them and is counted
    const bool done = mbar_wait_bounded(bar, 0u);
    if (__syncthreads_or(!done)) {
      if (threadIdx.x == 0) {
        atomicAdd(a.err + ERR_WAIT_TIMEOUT, 1ull);
        if (s_slot >= 0) atomicExch(a.st.claim + s_slot, 0u);
      }
      return;
    }
  }
  const SmemView<real> ebv{ EBs, g0[0] - R, g0[1], g0[2], G::WEX, G::WEX * G::WEY, G::NE };
  const int joff[3] = { ng + T0[0] - H::J_LO, ng + T0[1] - H::J_LO,
                        D == 3 ? ng + T0[2] - H::J_LO : 0 };
  const int jb      = -joff[0] - joff[1] * G::WJ0 - joff[2] * (G::WJ0 * G::WJ1);
  const int slot    = s_slot;
  // The thread's particle within each NT-particle chunk. With lane_stride
  // ls, ls consecutive warps share 32 ls consecutive particles, lane l of the
  // group's k-th warp taking particle ls l + k: each warp spans ls times as
  // many cells, so fewer of its lanes add to one J word, and the group
  // still reads whole lines.
  const int ls      = a.lane_stride;
  const int wid     = (int)(threadIdx.x >> 5);
  const int local   = (wid / ls) * (32 * ls) + ls * (int)(threadIdx.x & 31) + wid % ls;
  uint4*    recs    = slot >= 0 ? a.st.rec + (size_t)slot * a.st.cap * 2 : nullptr;
  // cell of a record relative to the tile: 8 bits per axis, offset by 64
  static_assert(G::TX + kDriftMargin + 2 < 64 && G::TY + kDriftMargin + 2 < 64 &&
                    G::TZ + kDriftMargin + 2 < 64,
                "record cells are 8-bit offsets from the tile origin");

  // 2. particles of the tile, species by species
  for (int s = 0; s < a.nsp; ++s) {
    const TiledSpecies<real>& S = a.s[s];
    real*          ux[3]  = { (real*)S.sp.ux1, (real*)S.sp.ux2, (real*)S.sp.ux3 };
    const real*    w      = (const real*)S.sp.w;
    int32_t*       ia[3]  = { S.sp.i1, S.sp.i2, S.sp.i3 };
    int32_t*       ipa[3] = { S.sp.i1p, S.sp.i2p, S.sp.i3p };
    float*         da[3]  = { S.sp.dx1, S.sp.dx2, S.sp.dx3 };
    float*         dpa[3] = { S.sp.dx1p, S.sp.dx2p, S.sp.dx3p };
    const int64_t  lo = S.tile_start[t], hi = S.tile_start[t + 1];
    for (int64_t p = lo + local; p < hi; p += NT) {
      Prtl<real> q;
      q.tag = S.sp.tag[p];
      if (q.tag != PIC_TAG_ALIVE) {
        if (q.tag != PIC_TAG_DEAD) atomicAdd(a.err + ERR_BAD_TAG, 1ull);
        continue;
      }
#pragma unroll
      for (int d = 0; d < D; ++d) {
        q.i[d]  = ia[d][p];
        q.dx[d] = da[d][p];
      }
      if (!cells_in_grid<D>(q.i, a.pc.n)) {
        atomicAdd(a.err + ERR_OUT_OF_GRID, 1ull);
        continue;
      }
      bool near = true, edge = false;
#pragma unroll
      for (int d = 0; d < D; ++d) {
        const int T = d == 0 ? G::TX : (d == 1 ? G::TY : G::TZ);
        near = near && (q.i[d] >= T0[d] - M) && (q.i[d] < T0[d] + T + M);
        // a stencil that can reach the ghost layers of a non-periodic axis is
        // deposited at the reference's coordinates: there the reference keeps
        // the raw ghost currents, unfolded along the periodic axes
        edge = edge || (!a.periodic[d] &&
                        (q.i[d] < H::J_LO - M + 1 || q.i[d] >= a.pc.n[d] - (H::J_HI - M) - 1));
      }
      {
        // particles that drifted past the margin, or whose stencil can reach
        // the ghost layers of a non-periodic axis, are left to the
        // per-particle kernel (global gathers, reference coordinates)
        const bool     defer = !near || edge;
        const unsigned ball  = __ballot_sync(__activemask(), defer);
        if (defer) {
          const int      lane   = threadIdx.x & 31;
          const int      leader = __ffs(ball) - 1;
          unsigned       base   = 0;
          if (lane == leader) base = atomicAdd(S.ovf_count, (unsigned)__popc(ball));
          base = __shfl_sync(ball, base, leader);
          S.ovf[base + __popc(ball & ((1u << lane) - 1u))] = (int32_t)p;
          continue;
        }
      }
#pragma unroll
      for (int d = 0; d < 3; ++d) q.u[d] = ux[d][p];
      real e0[3], b0[3];
      int  ic[3] = { q.i[0] + ng, q.i[1] + ng, D == 3 ? q.i[2] + ng : 0 };
      real dc[3] = { (real)q.dx[0], (real)q.dx[1], D == 3 ? (real)q.dx[2] : (real)0 };
      if constexpr (O == 0) interp_zigzag<D, real>(ebv, ic, dc, e0, b0);
      else                  interp_shape<D, O, real>(ebv, ic, dc, e0, b0);
#pragma unroll
      for (int d = 0; d < D; ++d) {
        e0[d] = e0[d] * a.dx;
        b0[d] = b0[d] * a.dx;
      }
      if (S.vay) vay<real>(S.ndth, q.u, e0, b0);
      else       boris<real>(S.ndth, q.u, e0, b0);
      move_and_bound<D, real>(q, true, a.dt, a.dx, a.pc);
#pragma unroll
      for (int d = 0; d < D; ++d) {
        ia[d][p] = q.i[d];
        da[d][p] = q.dx[d];
      }
#pragma unroll
      for (int d = 0; d < 3; ++d) ux[d][p] = q.u[d];
      if (q.tag != PIC_TAG_ALIVE) S.sp.tag[p] = q.tag;
      if (a.write_prev) {
#pragma unroll
        for (int d = 0; d < D; ++d) {
          ipa[d][p] = q.ip[d];
          dpa[d][p] = q.dxp[d];
        }
      }
      if (q.tag == PIC_TAG_DEAD || S.charge == (real)0) continue;
      // deposit at the coordinates before the periodic wrap (a shift of both
      // i and i_prev by n leaves every contribution unchanged up to the image
      // cell, which the flush folds back)
#pragma unroll
      for (int d = 0; d < D; ++d) {
        q.i[d] -= q.wrap[d];
        q.ip[d] -= q.wrap[d];
      }
      // in fixed point the weight carries the power-of-two scale, so every
      // contribution arrives scaled exactly (w 2^s rounds like w)
      const real wp = fixed ? w[p] * scale : w[p];
      // Shared-memory atomics serialise the lanes of a warp that hit one
      // word, and cell-sorted lanes share their boxes: odd and even lanes
      // add to separate copies, which halves those collisions. The flush
      // sums the copies' integer totals, so J is unchanged to the bit.
      unsigned* Jc  = Jw + (G::COPIES == 2 ? (int)(threadIdx.x & 1) * G::COPY : 0);
      auto      add = [&](int i, int j, int k, int c, real v) {
        const int e = jb + i + j * G::WJ0 + k * (G::WJ0 * G::WJ1) + c * G::NJ;
        if (fixed) FA::add(Jc + e, G::PLANE, v);
        else       atomicAdd(Jr + e, v);
      };
      if constexpr (G::STAGE) {
        if (recs) {
          // the 2D deposit reads the out-of-plane velocity, the 3D one none
          real vp[3] = { 0, 0, 0 };
          if constexpr (D == 2) deposit_velocity<D, real>(q, a.dx, vp);
          if (support_unmoved<D, O, real>(q)) {
            deposit_with_velocity<D, O, real, true>(q, vp, wp, S.charge, a.inv_dt, ng, nullptr,
                                                    add);
            continue;
          }
          // a record needs the move to stay within one cell per axis
          bool one = true;
#pragma unroll
          for (int d = 0; d < D; ++d) one = one && q.ip[d] - q.i[d] >= -1 && q.ip[d] - q.i[d] <= 1;
          const unsigned ball = __ballot_sync(__activemask(), one);
          if (one) {
            const int lane   = threadIdx.x & 31;
            const int leader = __ffs(ball) - 1;
            unsigned  base   = 0;
            if (lane == leader) base = atomicAdd(&s_nrec, (unsigned)__popc(ball));
            base             = __shfl_sync(ball, base, leader);
            const unsigned r = base + __popc(ball & ((1u << lane) - 1u));
            if (r < (unsigned)a.st.cap) {
              unsigned cells = 0;
#pragma unroll
              for (int d = 0; d < D; ++d)
                cells |= ((unsigned)(q.i[d] - T0[d] + 64) << (8 * d)) |
                         ((unsigned)(q.ip[d] - q.i[d] + 1) << (24 + 2 * d));
              const float coeff = (float)(wp * S.charge);
              // 3D: the offsets x3 in the third words; 2D: the out-of-plane
              // velocity in their place
              const float w3 = D == 3 ? q.dx[2] : (float)vp[2], p3 = D == 3 ? q.dxp[2] : 0.f;
              __stcg(recs + 2 * r, make_uint4(cells, __float_as_uint(q.dx[0]),
                                              __float_as_uint(q.dx[1]), __float_as_uint(w3)));
              __stcg(recs + 2 * r + 1,
                     make_uint4(__float_as_uint(q.dxp[0]), __float_as_uint(q.dxp[1]),
                                __float_as_uint(p3), __float_as_uint(coeff)));
              continue;
            }
          }
        }
      }
      deposit_particle<D, O, real>(q, wp, S.charge, a.inv_dt, a.dx, ng, nullptr, add);
    }
  }
  __syncthreads();
  if constexpr (G::STAGE) {
    // the recorded particles, 32 per warp; the record's coefficient is the
    // product weight * charge that the direct deposit forms, times charge 1
    if (recs) {
      const int nrec = min((int)s_nrec, a.st.cap);
      unsigned* Jc   = Jw + (G::COPIES == 2 ? (int)(threadIdx.x & 1) * G::COPY : 0);
      auto      add  = [&](int i, int j, int k, int c, real v) {
        const int e = jb + i + j * G::WJ0 + k * (G::WJ0 * G::WJ1) + c * G::NJ;
        if (fixed) FA::add(Jc + e, G::PLANE, v);
        else       atomicAdd(Jr + e, v);
      };
      for (int r = threadIdx.x; r < nrec; r += NT) {
        const uint4 u0 = __ldcg(recs + 2 * r), u1 = __ldcg(recs + 2 * r + 1);
        Prtl<real>  q;
        const float dx[3]  = { __uint_as_float(u0.y), __uint_as_float(u0.z), __uint_as_float(u0.w) };
        const float dxp[3] = { __uint_as_float(u1.x), __uint_as_float(u1.y), __uint_as_float(u1.z) };
        const real  vp[3]  = { 0, 0, D == 2 ? (real)dx[2] : (real)0 };
#pragma unroll
        for (int d = 0; d < D; ++d) {
          q.i[d]   = (int)((u0.x >> (8 * d)) & 255u) - 64 + T0[d];
          q.ip[d]  = q.i[d] + (int)((u0.x >> (24 + 2 * d)) & 3u) - 1;
          q.dx[d]  = dx[d];
          q.dxp[d] = dxp[d];
        }
        deposit_with_velocity<D, O, real>(q, vp, (real)__uint_as_float(u1.w), (real)1, a.inv_dt,
                                          ng, nullptr, add);
        // Lanes 4m..4m+3 have read the four records of one 128-byte line and
        // used them: the line is dropped from L2 unwritten, so the records
        // cost no DRAM traffic (the next CTA on this buffer writes before it
        // reads)
        const int      base = r - (int)(threadIdx.x & 31);
        const unsigned m    = nrec - base >= 32 ? 0xffffffffu : (1u << (nrec - base)) - 1u;
        __syncwarp(m);
        if ((r & 3) == 0) discard_l2_line(recs + 2 * r);
      }
    }
    __syncthreads();
    if (threadIdx.x == 0 && slot >= 0) atomicExch(a.st.claim + slot, 0u);
  }

  // 3. flush the J window (periodic images folded onto active cells)
  for (int idx = threadIdx.x; idx < 3 * G::NJ; idx += NT) {
    real      v = 0;
    long long units = 0;  // the entry in global units (exact accumulator)
    if (fixed) {
      long long t = 0;
      bool      any = false;
#pragma unroll
      for (int k = 0; k < G::COPIES; ++k) {
        const unsigned* wk = Jw + k * G::COPY + idx;
        if (FA::nonzero(wk, G::PLANE)) {
          any = true;
          t += FA::total(wk, G::PLANE);
        }
      }
      if (!any) continue;
      if (global_unit) units = (long long)((unsigned long long)t << (a.fj.bits - b));
      else             v = FA::to_real(t, unscale);
    } else {
      v = Jr[idx];
      if (v == (real)0) continue;
      if (global_unit) units = __float2ll_rn((float)v * ldexpf(1.f, a.fj.bits - ex));
    }
    int       r  = idx;
    const int wi = r % G::WJ0;
    r /= G::WJ0;
    const int wj = r % G::WJ1;
    r /= G::WJ1;
    const int wk = r % G::WJ2;
    const int c  = r / G::WJ2;
    int       gc[3] = { T0[0] - H::J_LO + wi, T0[1] - H::J_LO + wj,
                        D == 3 ? T0[2] - H::J_LO + wk : 0 };
    bool      inside = true;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      if (a.periodic[d]) {
        gc[d] = wrap_periodic(gc[d], a.pc.n[d]);
      } else if (gc[d] < -ng || gc[d] >= a.pc.n[d] + ng) {
        inside = false;
      }
    }
    if (inside) {
      if constexpr (sizeof(real) == 4) {
        if (global_unit) {
          a.fj.add_units(gc[0] + ng, gc[1] + ng, D == 3 ? gc[2] + ng : 0, c, units);
          continue;
        }
      }
      atomicAdd(a.J.p + a.J.idx(gc[0] + ng, gc[1] + ng, D == 3 ? gc[2] + ng : 0, c), v);
    } else {
      atomicAdd(a.err + ERR_STENCIL_OUT, 1ull);
    }
  }
}

template <int D, int O, typename real>
cudaError_t launch_push_deposit_tiled(const TiledArgs<real>& a, cudaStream_t s);

// tile shape of a build, for the host (sort key and tile count)
void tile_shape(int dim, int real_bytes, int order, int out[3]);

}  // namespace pic
