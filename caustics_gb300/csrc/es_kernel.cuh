// Extended-source magnification by contour integration, one CTA per source
// position, persistent over a list or a device work queue
// (src/caustics/extended_source.py:56-904, integrate.py:18-121).
//
// Phases inside a CTA (256 threads), all state in shared memory:
//  A  n0 = npts/2 limb points solved in parallel (cold start, one thread per
//     point); rows put in the order of the reference's sequential warm-start
//     chain: clear steps by nearest roots, ambiguous steps and the first point
//     by the reference's own iteration (refea, bit-exact) on lane groups (the
//     first point's, in the batched path, by es_first_order_kernel ahead of
//     this kernel);
//  B  10 refinement rounds: gap per interval = max over images |dz| where either
//     end is a real image, the n_add largest gaps (ties: larger index first, as
//     argsort(...)[::-1]) get a midpoint point (extended_source.py:109-135);
//     the intervals are ranked once and kept as a sorted list into which each
//     round merges its new intervals; new points solved in parallel steps
//     (coefficients per point; FP32 Aberth on a lane group per point; FP64
//     Newton and image filter per root; labelling per point against the left
//     neighbour, the reference's warm start);
//  C  final chained matching over all limb points (extended_source.py:150-151):
//     candidate rows sorted by distance in parallel, the greedy pass on one
//     warp (lane per track);
//  D  tracks -> closed tracks / split open segments (extended_source.py:156-309),
//     change points found in parallel;
//  E  segment linking into <= 3 contours (extended_source.py:312-727);
//  F  Green's-theorem integral: trapezoid (uniform) or the Dominik (1998) P/Q
//     line integrals with split Gauss-Legendre quadrature (integrate.py:47-121),
//     ld_group lanes per contour point, FP64 or FP32 (shifted lens equation)
//     nodes;
//  and with GRAD the hand-written adjoint of A-F (contours recomputed).
#pragma once
#include <type_traits>

#include "aberth.cuh"
#include "aberth_ref.cuh"
#include "dword.cuh"
#include "es.h"
#include "internal.h"

namespace cgb {

// Threads of a contour-kernel CTA: chosen at launch (128 or 256; 128 lets four
// CTAs share an SM where their shared memory allows, for more independent
// evaluations in the latency-bound phases); device code reads blockDim.x.
constexpr int ES_MAX_THREADS = 256;
constexpr int ES_MAX_WARPS = ES_MAX_THREADS / 32;
#define ES_THREADS ((int)blockDim.x)
#define ES_WARPS ((int)blockDim.x >> 5)
constexpr int MAX_SEG = 30;      // 3 * n_images for triple lenses
constexpr int MAX_PIECES = 24;   // 1 + up to 20 merges per contour
constexpr int N_CONTOURS = 3;    // merged contours (extended_source.py:871)
constexpr int MAX_CLOSED = 10;

struct Piece {
  int16_t t, l, r;  // track, [l, r) positions
  int16_t dir;      // +1 forward, -1 reversed
};

struct Segment {
  int16_t t, l, r;
  int16_t par;  // parity of the head point (+1 / -1), 0 for an empty segment
  double len;   // path length
  int alive;
};

struct MergeState {
  Segment seg[MAX_SEG];
  int order[MAX_SEG];
  int nseg;
  Piece pieces[N_CONTOURS][MAX_PIECES];
  int npieces[N_CONTOURS];
  int cpar[N_CONTOURS];
  int cnpts[N_CONTOURS];
  int closed_tracks[MAX_CLOSED];
  int nclosed;
  int all_closed;
  uint32_t flags;
};

// shared-memory layout for one CTA
template <int DEG>
struct EsSmem {
  cd *Z;          // [Lcap][DEG] roots per slot (rows)
  double *TH;     // [Lcap] theta per slot
  uint16_t *MK;   // [Lcap] real-image bits per slot (by row)
  uint16_t *PP;   // [Lcap] positive-parity bits per slot (by row)
  uint16_t *ZP;   // [Lcap] zero-det bits (parity 0)
  uint16_t *ORD;  // [Lcap] position -> slot
  uint16_t *ORD2;
  uint64_t *PERM; // [Lcap] packed 4-bit permutation: track -> row
  uint64_t *BMAP; // [Lcap] warm-start map of the limb chain: root of k-1 -> root of k
  uint64_t *USED; // [Lcap] chain order of k-1 the map was computed with
  uint64_t *CAND; // [Lcap * DEG] candidate rows of position k sorted by distance, per row of k-1
  cd *GG;         // [CPcap] adjoint: dT/dx_i + i dT/dy_i per contour point
  double *KEY;    // [Lcap]
  int *SCAN;      // [Lcap + 1]
  uint32_t *CP;   // [CPcap] contour points: slot * DEG + row
  MergeState *M;
};

__device__ __forceinline__ int perm_get(uint64_t p, int t) { return (int)((p >> (4 * t)) & 15u); }
__device__ __forceinline__ uint64_t perm_set(uint64_t p, int t, int v) {
  return (p & ~(15ull << (4 * t))) | ((uint64_t)v << (4 * t));
}

// greedy nearest matching of rows b against a (processing order = a's order):
// returns packed res[i] = b row matched to a[i]
template <int DEG>
__device__ uint64_t greedy_match(const cd *a, const cd *b) {
  uint32_t taken = 0;
  uint64_t res = 0;
  for (int i = 0; i < DEG; ++i) {
    int best = 0;
    double bd = INFINITY;
    bool found = false;
    for (int j = 0; j < DEG; ++j) {
      if ((taken >> j) & 1u) continue;
      double d = norm2(b[j] - a[i]);
      if (!found || d < bd) {
        bd = d;
        best = j;
        found = true;
      }
    }
    taken |= 1u << best;
    res = perm_set(res, i, best);
  }
  return res;
}

// nearest row of b for every row of a; ok = the map is injective (then the
// greedy result does not depend on the processing order)
template <int DEG>
__device__ uint64_t nearest_map(const cd *a, const cd *b, bool &ok) {
  uint64_t res = 0;
  uint32_t used = 0;
  ok = true;
  for (int i = 0; i < DEG; ++i) {
    int best = 0;
    double bd = norm2(b[0] - a[i]);
    for (int j = 1; j < DEG; ++j) {
      double d = norm2(b[j] - a[i]);
      if (d < bd) {
        bd = d;
        best = j;
      }
    }
    if ((used >> best) & 1u) ok = false;
    used |= 1u << best;
    res = perm_set(res, i, best);
  }
  return res;
}

// block-wide exclusive scan of SCAN[0..n) in place; returns the total
static __device__ int block_exclusive_scan(int *buf, int n, int *warp_tot) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int carry = 0;
  for (int base = 0; base < n; base += ES_THREADS) {
    int i = base + tid;
    int v = i < n ? buf[i] : 0;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
      int t = lane < ES_WARPS ? warp_tot[lane] : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += y;
      }
      if (lane < ES_WARPS) warp_tot[lane] = t;
    }
    __syncthreads();
    int off = (warp > 0 ? warp_tot[warp - 1] : 0) + carry;
    if (i < n) buf[i] = off + x - v;
    int tot = warp_tot[ES_WARPS - 1];
    __syncthreads();
    carry += tot;
  }
  return carry;
}

// Deterministic accumulation of per-lane values into per-key slots: acc[key]
// += v for every lane with key >= 0, where the keys of a warp's lanes form
// contiguous runs (a contour's points are consecutive).  Each run is summed by
// a fixed shuffle tree and its first lane adds the total (one writer per run;
// the runs of one warp have distinct keys, and a warp's calls follow program
// order), so the result does not depend on scheduling.  All 32 lanes call.
__device__ __forceinline__ void warp_run_add(int key, double v, double *acc, int stride = 1) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const double u = __shfl_down_sync(0xffffffffu, v, o);
    const int ku = __shfl_down_sync(0xffffffffu, key, o);
    if (lane + o < 32 && ku == key) v += u;
  }
  const int kp = __shfl_up_sync(0xffffffffu, key, 1);
  if (key >= 0 && (lane == 0 || kp != key)) acc[key * stride] += v;
}

// Length of the limb interval between slots s1 and s2 for the refinement
// (extended_source.py:110-113): the largest |z2 - z1| over the rows that are a
// real image at either end, taken as sqrt of the largest squared distance
// (sqrt is monotone and correctly rounded).
template <int DEG>
__device__ __forceinline__ double interval_len(const EsSmem<DEG> &S, int s1, int s2) {
  const cd *a = S.Z + (size_t)s1 * DEG, *b = S.Z + (size_t)s2 * DEG;
  const uint16_t m = S.MK[s1] | S.MK[s2];
  double g2 = 0.0;
  for (int i = 0; i < DEG; ++i)
    if ((m >> i) & 1u) g2 = fmax(g2, norm2(b[i] - a[i]));
  return sqrt(g2);
}

// Bitonic sort of n (a power of two) pairs (v, ix) into descending order of v,
// equal v by descending ix; every thread of the block calls it after a block
// barrier.  Thread t owns compare-exchange t (plus multiples of the block size)
// of each stage, so at strides up to 32 a warp's exchanges stay inside its own
// 64-element blocks: two consecutive such stages need only the warp to
// synchronise, while a stage next to a wider one synchronises the block.
static __device__ void bitonic_sort_desc(long long *v, uint16_t *ix, int n) {
  int prev = 0;
  for (int size = 2; size <= n; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      if (stride > 32 || prev > 32)
        __syncthreads();
      else
        __syncwarp();
      prev = stride;
      for (int t = threadIdx.x; t < (n >> 1); t += ES_THREADS) {
        const int i = 2 * stride * (t / stride) + (t & (stride - 1)), j = i + stride;
        const long long a = v[i], b = v[j];
        const uint16_t ia = ix[i], ib = ix[j];
        const bool b_first = (b > a) || (b == a && ib > ia);  // b precedes a in the final order
        if (b_first == ((i & size) == 0)) {
          v[i] = b;
          v[j] = a;
          ix[i] = ib;
          ix[j] = ia;
        }
      }
    }
  }
  __syncthreads();
}

// EARLY: the mixed solver's polish may stop after one step (aberth_mixed);
// the forward kernels take it, the adjoint keeps full FP64 roots (its image
// tangents ~1/det J amplify root errors near critical curves: 1e-13 roots
// moved a curve's gradient by 1e-3)
template <int NL, int PREC, bool EARLY = false>
__device__ void solve_limb_point(const EsParams &P, const EsItem &I, double th, cd *zrow, const cd *warm,
                                 uint16_t &mkb, uint16_t &pp, uint16_t &zp, uint32_t &flags) {
  constexpr int DEG = NL * NL + 1;
  double s, c;
  sincos(th, &s, &c);
  cd w = mk(__dadd_rn(__dmul_rn(I.rho, c), I.w0.x), __dadd_rn(__dmul_rn(I.rho, s), I.w0.y));
  cd p[DEG + 1], z[DEG];
  lens_poly<NL>(I.L, w, p);
  if (warm) {
#pragma unroll
    for (int i = 0; i < DEG; ++i) z[i] = warm[i] + mk(1e-6 * ((i & 1) ? 0.5 : -0.5), 1e-6 * ((i & 2) ? 0.5 : -0.5));
  }
  int it = (PREC == MIXED) ? aberth_mixed<DEG, true, EARLY>(p, z, P.itmax, warm != nullptr, flags)
                           : aberth64<DEG>(p, z, P.itmax, warm != nullptr);
  if (it < 0) flags |= CGB_ST_NOCONV;
  mkb = 0;
  pp = 0;
  zp = 0;
#pragma unroll
  for (int i = 0; i < DEG; ++i) {
    zrow[i] = z[i];
    double r, d;
    lens_filter<NL>(I.L, z[i], w, r, d);
    if (r < 1e-6) mkb |= 1u << i;
    if (r > 1e-6 / 30 && r < 1e-6 * 30) flags |= CGB_ST_AMBIGUOUS;
    if (d > 0) pp |= 1u << i;
    if (d == 0) zp |= 1u << i;
  }
}

// Step map between consecutive limb points (raw rows of k-1 -> raw rows of k).
// When every root of k-1 has a successor clearly nearer than any other root
// (d1 < d2/2, and no two share one) a warm-started Aberth iteration lands each
// iterate on that nearest root whatever the arithmetic, so the map is final.
// Otherwise the step is ambiguous and the returned greedy map is only a guess.
template <int DEG>
__device__ uint64_t step_map(const cd *a, const cd *b, bool &ambiguous) {
  uint64_t res = 0;
  uint32_t used = 0;
  ambiguous = false;
  // squared distances are >= +0: compared as their bit patterns (unsigned,
  // any NaN above +inf) on the integer pipe
  for (int i = 0; i < DEG; ++i) {
    unsigned long long d1 = (unsigned long long)__double_as_longlong(INFINITY), d2 = d1;
    int best = 0;
    for (int j = 0; j < DEG; ++j) {
      const unsigned long long d = (unsigned long long)__double_as_longlong(norm2(b[j] - a[i]));
      if (d < d1) {
        d2 = d1;
        d1 = d;
        best = j;
      } else if (d < d2) {
        d2 = d;
      }
    }
    if (!(__longlong_as_double((long long)d1) < 0.25 * __longlong_as_double((long long)d2)) || ((used >> best) & 1u))
      ambiguous = true;
    used |= 1u << best;
    res = perm_set(res, i, best);
  }
  return ambiguous ? greedy_match<DEG>(a, b) : res;
}

// Which root of limb point k each root of point k-1 reaches when the reference
// warm-starts point k from point k-1 with rows in order `prev` (track -> raw row
// of k-1), computed with the reference's arithmetic (point_source.py:1711-1759,
// extended_source.py:79-98): warm_map_ref_group.  jitter adds the warm-start
// perturbation of the refinement solves.  Returns the map raw root of k-1 ->
// raw root of k.  first_point_order_group labels the first limb point's roots
// as the reference's cold start from its real-valued initial guesses produces
// them: track t -> raw row.
// Lanes that share one faithful solve (one lane per root).
template <int DEG>
struct RefGroup {
  static constexpr int G = DEG <= 8 ? 8 : 16;
};

// warm_map_ref / first_point_order on a group of RefGroup<DEG>::G lanes that
// call together (refea::solve_group); every lane returns the map.
template <int NL>
__device__ uint64_t warm_map_ref_group(const EsParams &P, const EsItem &I, double th, const cd *zprev, uint64_t prev,
                                       const cd *zcur, bool jitter, int &iters) {
  constexpr int DEG = NL * NL + 1, G = RefGroup<DEG>::G;
  const int lane = threadIdx.x & 31, r = lane & (G - 1);
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (lane - r));
  double s, c;
  sincos(th, &s, &c);
  cd p[DEG + 1];
  lens_poly<NL>(I.L, mk(__dadd_rn(__dmul_rn(I.rho, c), I.w0.x), __dadd_rn(__dmul_rn(I.rho, s), I.w0.y)), p);
  cd zr = mk(0.0, 0.0);
  if (r < DEG) {
    zr = zprev[perm_get(prev, r)];
    if (jitter) zr = zr + mk(1e-6 * ((r & 1) ? 0.5 : -0.5), 1e-6 * ((r & 2) ? 0.5 : -0.5));
  }
  iters = refea::solve_group<DEG, G>(p, zr, P.itmax, true, zcur);
  cd z[DEG];
#pragma unroll
  for (int t = 0; t < DEG; ++t) z[t] = refea::gshfl<G>(gmask, zr, t);
  const uint64_t rowmap = greedy_match<DEG>(z, zcur);  // iterate t -> raw root of k
  uint64_t nb = 0;
  for (int t = 0; t < DEG; ++t) nb = perm_set(nb, perm_get(prev, t), perm_get(rowmap, t));
  return nb;
}

template <int NL, int G = RefGroup<NL * NL + 1>::G>
__device__ uint64_t first_point_order_group(const EsParams &P, const EsItem &I, double th, const cd *zraw,
                                            int &iters) {
  constexpr int DEG = NL * NL + 1;
  const unsigned gmask = refea::gmask_of<G>();
  double s, c;
  sincos(th, &s, &c);
  cd p[DEG + 1];
  lens_poly<NL>(I.L, mk(__dadd_rn(__dmul_rn(I.rho, c), I.w0.x), __dadd_rn(__dmul_rn(I.rho, s), I.w0.y)), p);
  cd zr = mk(0.0, 0.0);
  iters = refea::solve_group<DEG, G>(p, zr, P.itmax, false, zraw);
  cd z[DEG];
#pragma unroll
  for (int t = 0; t < DEG; ++t) z[t] = refea::gshfl<G>(gmask, zr, t);
  return greedy_match<DEG>(z, zraw);
}

// permute the rows of one slot in place: new row t = old row perm[t]
template <int DEG>
__device__ void apply_rows(cd *zrow, uint16_t &mkb, uint16_t &pp, uint16_t &zp, uint64_t perm) {
  cd tmp[DEG];
  uint16_t m2 = 0, p2 = 0, z2 = 0;
  for (int t = 0; t < DEG; ++t) tmp[t] = zrow[t];
  for (int t = 0; t < DEG; ++t) {
    int r = perm_get(perm, t);
    zrow[t] = tmp[r];
    m2 |= ((mkb >> r) & 1u) << t;
    p2 |= ((pp >> r) & 1u) << t;
    z2 |= ((zp >> r) & 1u) << t;
  }
  mkb = m2;
  pp = p2;
  zp = z2;
}

// Chained greedy matching over positions [0, n) of ORD (utils.py:15-40 applied
// along the limb, extended_source.py:34-53); writes PERM[k] = track -> row.
// In parallel, every row of position k-1 gets its candidate rows of position k
// sorted by distance (stable, 4 bits each).  The sequential pass then runs on
// one warp, lane t holding track t's row: when the tracks' first candidates
// are all different, each track takes its own (what the greedy order gives
// whenever nothing collides); otherwise the tracks pick in track order, each
// its first untaken candidate.
template <int DEG>
__device__ void chain_match(EsSmem<DEG> &S, int n) {
  const int tid = threadIdx.x;
  for (int idx = tid; idx < (n - 1) * DEG; idx += ES_THREADS) {
    const int k = 1 + idx / DEG, i = idx % DEG;
    const cd a = S.Z[(size_t)S.ORD[k - 1] * DEG + i];
    const cd *b = S.Z + (size_t)S.ORD[k] * DEG;
    long long d[DEG];  // squared distances are >= +0: their bit patterns order as integers
    int o[DEG];
    for (int j = 0; j < DEG; ++j) {
      d[j] = __double_as_longlong(norm2(b[j] - a));
      o[j] = j;
    }
    for (int j = 1; j < DEG; ++j)  // stable insertion sort
      for (int m = j; m > 0 && d[o[m]] < d[o[m - 1]]; --m) {
        int x = o[m];
        o[m] = o[m - 1];
        o[m - 1] = x;
      }
    uint64_t packed = 0;
    for (int j = 0; j < DEG; ++j) packed = perm_set(packed, j, o[j]);
    S.CAND[(size_t)k * DEG + i] = packed;
  }
  __syncthreads();
  if (tid < 32) {
    const unsigned full = 0xffffffffu;
    const int t = tid;
    const bool own = t < DEG;
    int row = t;  // PERM[0] is the identity
    if (t == 0) {
      uint64_t ident = 0;
      for (int q = 0; q < DEG; ++q) ident = perm_set(ident, q, q);
      S.PERM[0] = ident;
    }
    for (int k = 1; k < n; ++k) {
      const uint64_t cand = own ? S.CAND[(size_t)k * DEG + row] : 0ull;
      const int c0 = (int)(cand & 15u);
      const unsigned firsts = __reduce_or_sync(full, own ? 1u << c0 : 0u);
      if (__popc(firsts) == DEG) {
        row = c0;
      } else {
        unsigned taken = 0;
        for (int tt = 0; tt < DEG; ++tt) {
          int pick = 0;
          if (t == tt)
            for (int j = 0; j < DEG; ++j) {
              const int c = perm_get(cand, j);
              if (!((taken >> c) & 1u)) {
                pick = c;
                break;
              }
            }
          pick = __shfl_sync(full, pick, tt);
          taken |= 1u << pick;
          if (t == tt) row = pick;
        }
      }
      const uint64_t word = own ? (uint64_t)row << (4 * t) : 0ull;
      const unsigned lo = __reduce_or_sync(full, (unsigned)word), hi = __reduce_or_sync(full, (unsigned)(word >> 32));
      if (t == 0) S.PERM[k] = ((uint64_t)hi << 32) | lo;
    }
  }
  __syncthreads();
}

// ---- merging helpers (single thread) ----
template <int DEG>
struct TrackView {
  const EsSmem<DEG> *S;
  __device__ cd at(int t, int k) const {
    int slot = S->ORD[k];
    int row = perm_get(S->PERM[k], t);
    return S->Z[(size_t)slot * DEG + row];
  }
  __device__ uint32_t cp(int t, int k) const {
    int slot = S->ORD[k];
    return (uint32_t)(slot * DEG + perm_get(S->PERM[k], t));
  }
};

// point i of a piece list (0 beyond the end, like the zero padding)
template <int DEG>
__device__ cd pieces_point(const TrackView<DEG> &V, const Piece *pc, int np, int i, int cap) {
  if (i < 0) i += cap;  // negative index wraps (JAX/NumPy), lands in the zero padding
  for (int q = 0; q < np; ++q) {
    int n = pc[q].r - pc[q].l;
    if (i < n) return V.at(pc[q].t, pc[q].dir > 0 ? pc[q].l + i : pc[q].r - 1 - i);
    i -= n;
  }
  return mk(0, 0);
}

// the two points defining a segment end (extended_source.py:373-393)
template <int DEG>
__device__ void end_line(const TrackView<DEG> &V, const Piece *pc, int np, int tidx, bool head, int cap, cd &l0,
                         cd &l1) {
  if (head) {
    cd x0 = pieces_point(V, pc, np, 0, cap), x1 = pieces_point(V, pc, np, 1, cap);
    if (cabs(x1 - x0) > 1e-5 || tidx <= 1) {
      l0 = x1;
      l1 = x0;
    } else {
      l0 = pieces_point(V, pc, np, 2, cap);
      l1 = x1;
    }
  } else {
    cd xt = pieces_point(V, pc, np, tidx, cap), xm = pieces_point(V, pc, np, tidx - 1, cap);
    int s0 = (cabs(xt - xm) > 1e-5 || tidx <= 1) ? tidx - 1 : tidx - 2;
    s0 = min(max(s0, 0), cap - 2);
    l0 = pieces_point(V, pc, np, s0, cap);
    l1 = pieces_point(V, pc, np, s0 + 1, cap);
  }
}

// _connection_condition (extended_source.py:324-442)
template <int DEG>
__device__ bool connect_ok(const TrackView<DEG> &V, const Piece *pa, int npa, int ta, int para, const Piece *pb,
                           int npb, int tb, int parb, int ctype, int cap) {
  bool same = (double)para * (double)parb > 0.0;
  bool cond_par = ctype < 2 ? same : !same;
  cd a0, a1, b0, b1;
  bool ahead = (ctype == 1 || ctype == 2), bhead = (ctype == 0 || ctype == 2);
  end_line(V, pa, npa, ta, ahead, cap, a0, a1);
  end_line(V, pb, npb, tb, bhead, cap, b0, b1);
  double dist = cabs(a1 - b1);
  cd v1 = a1 - a0, v2 = b1 - b0;
  double n1 = cabs(v1), n2 = cabs(v2);
  v1 = mk(v1.x / n1, v1.y / n1);
  v2 = mk(v2.x / n2, v2.y / n2);
  double ang = acos(v1.x * v2.x + v1.y * v2.y);
  bool c1 = dist < 1e-1;
  bool c2 = (180.0 - ang * (180.0 / 3.14159265358979323846)) < 60.0;
  bool c3 = cabs(a1 - b1) < cabs(a0 - b0);
  return cond_par && ((c1 && c2 && c3) || dist < 1e-5);
}

template <int DEG>
__device__ void merge_segments(EsSmem<DEG> &S, int L) {
  MergeState &M = *S.M;
  TrackView<DEG> V{&S};
  const int cap = 4 * L;  // padded length of the reference's merge arrays
  int cur[MAX_SEG], ncur = M.nseg;
  for (int i = 0; i < ncur; ++i) cur[i] = i;
  int maxsteps = 20;
  for (int c = 0; c < N_CONTOURS; ++c) {
    // stable sort by length, zero length (NaN in the reference) last
    int tmp[MAX_SEG], nt = 0;
    for (int i = 0; i < ncur; ++i) {
      const Segment &s = M.seg[cur[i]];
      if (s.alive && s.len != 0.0) {
        int j = nt;
        while (j > 0) {
          const Segment &o = M.seg[tmp[j - 1]];
          if (o.len > s.len) {
            tmp[j] = tmp[j - 1];
            --j;
          } else
            break;
        }
        tmp[j] = cur[i];
        ++nt;
      }
    }
    for (int i = 0; i < ncur; ++i) {
      const Segment &s = M.seg[cur[i]];
      if (!(s.alive && s.len != 0.0)) tmp[nt++] = cur[i];
    }
    // active segment
    Piece *pa = M.pieces[c];
    int npa = 0, ta = 0, para = 0;
    {
      const Segment &s = M.seg[tmp[0]];
      if (s.alive) {
        pa[0] = Piece{s.t, s.l, s.r, 1};
        npa = 1;
        ta = s.r - s.l - 1;
        para = s.par;
      }
    }
    int rest[MAX_SEG], nrest = ncur - 1;
    for (int i = 1; i < ncur; ++i) rest[i - 1] = tmp[i];
    for (int step = 0; step < maxsteps; ++step) {
      bool any = false;
      for (int i = 0; i < nrest; ++i) any |= (M.seg[rest[i]].alive != 0);
      if (!any) continue;
      cd ah = pieces_point(V, pa, npa, 0, cap), at = pieces_point(V, pa, npa, ta, cap);
      // four smallest of the 4 x nrest distances, ties by flattened index
      double bd[4];
      int bi[4];
      for (int q = 0; q < 4; ++q) {
        bd[q] = INFINITY;
        bi[q] = 1 << 30;
      }
      for (int ct = 0; ct < 4; ++ct)
        for (int i = 0; i < nrest; ++i) {
          const Segment &s = M.seg[rest[i]];
          cd bh = mk(0, 0), bt = mk(0, 0);
          if (s.alive) {
            bh = V.at(s.t, s.l);
            bt = V.at(s.t, s.r - 1);
          }
          cd pa_ = (ct == 0 || ct == 3) ? at : ah;
          cd pb_ = (ct == 0 || ct == 2) ? bh : bt;
          double d = cabs(pa_ - pb_);
          int f = ct * nrest + i;
          // insert into the sorted top-4 (strictly smaller, or equal with smaller index)
          for (int q = 0; q < 4; ++q) {
            if (d < bd[q] || (d == bd[q] && f < bi[q]) || (isnan(d) && false)) {
              for (int u = 3; u > q; --u) {
                bd[u] = bd[u - 1];
                bi[u] = bi[u - 1];
              }
              bd[q] = d;
              bi[q] = f;
              break;
            }
          }
        }
      int chosen = -1, cht = 0;
      for (int q = 0; q < 4 && chosen < 0; ++q) {
        if (bi[q] >= (1 << 30)) continue;
        int ct = bi[q] / nrest, i = bi[q] % nrest;
        const Segment &s = M.seg[rest[i]];
        Piece pb{s.t, s.l, s.r, 1};
        int npb = s.alive ? 1 : 0, tb = s.alive ? s.r - s.l - 1 : 0, parb = s.alive ? s.par : 0;
        if (connect_ok(V, pa, npa, ta, para, &pb, npb, tb, parb, ct, cap)) {
          chosen = i;
          cht = ct;
        }
      }
      if (chosen < 0) continue;
      Segment &s = M.seg[rest[chosen]];
      if (!s.alive || npa + 1 > MAX_PIECES) {
        M.flags |= CGB_ST_MERGE;
        continue;
      }
      Piece pb{s.t, s.l, s.r, 1};
      int nb = s.r - s.l;
      if (cht == 0) {  // T-H: A then B
        pa[npa++] = pb;
      } else if (cht == 1) {  // H-T: B then A
        for (int u = npa; u > 0; --u) pa[u] = pa[u - 1];
        pa[0] = pb;
        ++npa;
        para = s.par;
      } else if (cht == 2) {  // H-H: reversed B (parity flipped) then A
        for (int u = npa; u > 0; --u) pa[u] = pa[u - 1];
        pa[0] = Piece{s.t, s.l, s.r, -1};
        ++npa;
        para = -s.par;
      } else {  // T-T: A then reversed B
        pa[npa++] = Piece{s.t, s.l, s.r, -1};
      }
      ta = ta + nb;  // t1 + t2 + 1
      if (ta + 1 > cap) M.flags |= CGB_ST_MERGE;
      s.alive = 0;
    }
    M.npieces[c] = npa;
    M.cpar[c] = para;
    M.cnpts[c] = npa > 0 ? ta + 1 : 0;
    maxsteps -= 2;
    ncur = nrest;
    for (int i = 0; i < nrest; ++i) cur[i] = rest[i];
  }
  for (int i = 0; i < ncur; ++i)
    if (M.seg[cur[i]].alive) M.flags |= CGB_ST_MERGE;
}

// ---- Gauss-Legendre line integrals of the limb-darkened brightness ----
__device__ __forceinline__ double brightness_b(double r) {
  return r <= 1.0 ? 1.0 + sqrt(fmax(1.0 - r * r, 0.0)) : 1.0 - sqrt(fmax(1.0 - 1.0 / (r * r), 0.0));
}
// split points of integrate.py:49-64
__device__ __forceinline__ double split_point(double a, double b, double rho) {
  double absd = fabs(b - a);
  double sp = b > a ? b - 2 * rho : b + 2 * rho;
  return 0.5 * absd <= 2 * rho ? a + 0.5 * absd : sp;
}

// (P_i, Q_i) of one contour point (one thread), where
// P_i = -1/2 int_{y0}^{y_i} I(x_i, y) dy and Q_i = 1/2 int_{x0}^{x_i} I(x, y_i) dx,
// each split at the reference's split point into two Gauss-Legendre pieces.
// The node loop is uniform across the warp, so node tables are broadcast.
template <int NL>
__device__ cd ld_point_fp64(const EsParams &P, const EsItem &It, cd zc, cd z0, int j0, int jstep) {
  const double c0 = 3.0 / (3.0 - It.u1), u1 = It.u1, inv_rho = 1.0 / It.rho;
  const cd w0 = It.w0;
  double acc[2] = {0.0, 0.0};
#pragma unroll
  for (int isQ = 0; isQ < 2; ++isQ) {
    const double a = isQ ? z0.x : z0.y, b = isQ ? zc.x : zc.y;
    const double sp = split_point(a, b, It.rho);
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const double lo = half ? sp : a, hi = half ? b : sp;
      const double hw = 0.5 * (hi - lo), mid = 0.5 * (hi + lo);
      const int n = half ? P.n2 : P.n1;
      double sum = 0.0;
      for (int j = j0; j < n; j += jstep) {
        const double xn = fma(hw, P.gl_x[half][j], mid);
        cd zn = isQ ? mk(xn, zc.y) : mk(zc.x, xn);
        double r = cabs(lens_eq<NL>(It.L, zn) - w0) * inv_rho;
        double I = c0 * (u1 * brightness_b(r) + 1.0 - 2.0 * u1);
        sum = fma(P.gl_w[half][j], I, sum);
      }
      acc[isQ] += hw * sum;
    }
  }
  return mk(-0.5 * acc[0], 0.5 * acc[1]);  // (P_i, Q_i)
}

// Node arithmetic of the FP32 quadrature: approximate reciprocal (at most 2
// ulp, one special-function instruction) and square root through rsqrt; each
// node's FP32 value carries ~1e-7 relative error either way.
__device__ __forceinline__ cf crecip_fast(cf b) {
  const float inv = __fdividef(1.0f, b.x * b.x + b.y * b.y);
  return cf{b.x * inv, -b.y * inv};
}
// B(r) of the brightness profile from n = r^2 with one rsqrt:
//   r <= 1: 1 + sqrt(1 - n);  r > 1: 1 - sqrt(1 - 1/n) = 1 - a rsqrt(a n), a = n - 1.
__device__ __forceinline__ float brightness_bn_fast(float n) {
  const bool inside = n <= 1.0f;
  const float a = inside ? 1.0f - n : n - 1.0f;
  const float sq = a > 0.0f ? a * rsqrtf(inside ? a : a * n) : 0.0f;
  return inside ? 1.0f + sq : 1.0f - sq;
}

// FP32 nodes on a shifted lens equation:
//   lens_eq(zc + d) - w0 = (lens_eq(zc) - w0) + d + sum_j eps_j conj(d) / (D_j (D_j + conj(d))),
//   D_j = conj(zc) - conj(r_j);
// the FP64 prologue (once per point) provides every difference, so each FP32
// quantity is small relative to its own scale.
// Per-evaluation constants of the FP32 quadrature.
struct LdConst {
  float c0, u1, irf;
  float ej[3];  // eps_j / rho
};

template <int NL>
__device__ __forceinline__ LdConst ld_const(const EsItem &It) {
  LdConst k;
  const double inv_rho = 1.0 / It.rho;
  k.c0 = (float)(3.0 / (3.0 - It.u1));
  k.u1 = (float)It.u1;
  k.irf = (float)inv_rho;
#pragma unroll
  for (int j = 0; j < NL; ++j) k.ej[j] = (float)(It.L.eps[j] * inv_rho);
  return k;
}

// th: the limb angle of the contour point's limb point.  zc is an image of
// w0 + rho e^{i th}, so (lens_eq(zc) - w0) / rho = e^{i th} up to the root's
// residual (~1e-15), far below the FP32 node arithmetic.
// glf: FP32 copies of the Gauss-Legendre tables in shared memory,
// [half][0: nodes, 1: weights][j] (the conversions, once per block, are the
// ones the node loop would otherwise do per node).
template <int NL>
__device__ cd ld_point_mixed(const EsParams &P, const EsItem &It, const LdConst &K, cd zc, double th, cd z0, int j0,
                             int jstep, const float (*glf)[4][GL_MAX]) {
  // I = c0 (u1 B + 1 - 2 u1) = cu B + cc
  const float cu = K.c0 * K.u1, cc = K.c0 * (1.0f - 2.0f * K.u1);
  cf uc;
  sincosf((float)th, &uc.y, &uc.x);
  // D = conj(zc) - conj(r_j) in FP64 (an image near a lens makes it a small
  // difference of O(1) numbers), then FP32 like the nodes: on GB300 every FP64
  // instruction, conversions included, costs a warp the same ~64 cycles of its
  // scheduler's FP64 pipe
  cf Dj[NL], Dj2[NL];
  float ej[NL];
#pragma unroll
  for (int j = 0; j < NL; ++j) {
    const cd d = conj(zc) - conj(It.L.r[j]);
    Dj[j] = tof(d);
    Dj2[j] = Dj[j] * Dj[j];
    ej[j] = K.ej[j];
  }
  const float irf = K.irf;
  float acc[2] = {0.0f, 0.0f};
#pragma unroll
  for (int isQ = 0; isQ < 2; ++isQ) {
    const double a = isQ ? z0.x : z0.y, b = isQ ? zc.x : zc.y;
    const double sp = split_point(a, b, It.rho);
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const double lo = half ? sp : a, hi = half ? b : sp;
      const float lo_r = (float)(lo - b), hi_r = (float)(hi - b);  // relative to the contour point
      const float hw = 0.5f * (hi_r - lo_r), mid = 0.5f * (hi_r + lo_r);
      const int n = half ? P.n2 : P.n1;
      // |s|^2 at one node, s = (lens_eq(zc + delta) - w0) / rho; binary lenses
      // share one reciprocal between the two lens terms
      auto node_n2 = [&](float d) {
        const cf cdl = isQ ? mkf(d, 0.0f) : mkf(0.0f, -d);
        cf sacc = isQ ? mkf(fmaf(d, irf, uc.x), uc.y) : mkf(uc.x, fmaf(d, irf, uc.y));
        if constexpr (NL == 2) {
          const cf den0 = cfma(Dj[0], cdl, Dj2[0]), den1 = cfma(Dj[1], cdl, Dj2[1]);  // D (D + conj(delta))
          const float n0 = den0.x * den0.x + den0.y * den0.y, n1 = den1.x * den1.x + den1.y * den1.y;
          const float inv = __fdividef(1.0f, n0 * n1);
          const float i0 = ej[0] * inv * n1, i1 = ej[1] * inv * n0;
          const cf t0 = cdl * cf{den0.x * i0, -den0.y * i0}, t1 = cdl * cf{den1.x * i1, -den1.y * i1};
          sacc = sacc + t0 + t1;
        } else {
#pragma unroll
          for (int k = 0; k < NL; ++k) {
            const cf den = cfma(Dj[k], cdl, Dj2[k]);  // D (D + conj(delta))
            sacc = sacc + (cdl * crecip_fast(den)) * ej[k];
          }
        }
        return sacc.x * sacc.x + sacc.y * sacc.y;
      };
      // two nodes in flight per lane: independent chains for the in-order pipeline
      float s0 = 0.0f, s1 = 0.0f;
      int j = j0;
      for (; j + jstep < n; j += 2 * jstep) {
        const float n0 = node_n2(fmaf(hw, glf[half][0][j], mid));
        const float n1 = node_n2(fmaf(hw, glf[half][0][j + jstep], mid));
        s0 = fmaf(glf[half][1][j], fmaf(cu, brightness_bn_fast(n0), cc), s0);
        s1 = fmaf(glf[half][1][j + jstep], fmaf(cu, brightness_bn_fast(n1), cc), s1);
      }
      if (j < n) s0 = fmaf(glf[half][1][j], fmaf(cu, brightness_bn_fast(node_n2(fmaf(hw, glf[half][0][j], mid))), cc), s0);
      // FP32: the halves cancel by at most a factor 2 (the reference's split
      // point a + |b - a| / 2 can lie beyond a when b < a)
      acc[isQ] = fmaf(hw, s0 + s1, acc[isQ]);
    }
  }
  return mk(-0.5 * (double)acc[0], 0.5 * (double)acc[1]);  // (P_i, Q_i)
}


// ---- adjoint of the contour integral (binary lenses) ----
// Derivatives of one contour point's P_i / Q_i (integrate.py:49-109) with
// respect to its own position, the contour centroid coordinate, and the
// parameters (rho, u1, Re w0, Im w0, a, e1), differentiating through the node
// positions, the split point and the brightness profile exactly as the
// discretised integral depends on them.
// Parameter directions of the adjoint: rho, u1, Re w0, Im w0, then the lens:
// binary (a, e1): lenses at +-a with masses e1, 1 - e1; triple (a, e1, e2,
// Re r3, Im r3): masses e1, e2, 1 - e1 - e2 at a, -a, r3.
template <int NL>
struct GradDirs {
  static constexpr int NLENS = NL == 2 ? 2 : 5;
  static constexpr int NK = 4 + NLENS;
};
constexpr int NK_MAX = 9;

template <int NK>
struct PQGrad {
  double P, Q;
  double Px, Py, Pa;  // dP/dx_i, dP/dy_i, dP/dy0
  double Qx, Qy, Qa;  // dQ/dx_i, dQ/dy_i, dQ/dx0
  double Pk[NK], Qk[NK];  // the parameter directions (GradDirs)
};

enum { GK_RHO = 0, GK_U1 = 1, GK_WX = 2, GK_WY = 3, GK_A = 4, GK_E1 = 5, GK_E2 = 6, GK_R3X = 7, GK_R3Y = 8 };

// d lens_eq / d theta at a fixed image position for the lens directions,
// from u_j = 1 / (conj(z) - conj(r_j)): d/d eps_j = -u_j, d/d conj(r_j) =
// -eps_j u_j^2 (lens_eq = z - sum_j eps_j / (conj(z) - conj(r_j))).
template <int NL, typename R, typename C>
__device__ __forceinline__ void lens_shifts(const C (&u)[NL], const R (&ej)[NL], C (&ds)[GradDirs<NL>::NLENS]) {
  const C fa = u[0] * u[0] * ej[0] - u[1] * u[1] * ej[1];
  ds[0] = C{-fa.x, -fa.y};  // a: r_0 = a, r_1 = -a
  if constexpr (NL == 2) {
    ds[1] = u[1] - u[0];  // e1: eps_0 = e1, eps_1 = 1 - e1
  } else {
    ds[1] = u[2] - u[0];  // e1: eps_0 = e1, eps_2 = 1 - e1 - e2
    ds[2] = u[2] - u[1];  // e2: eps_1 = e2, eps_2 = 1 - e1 - e2
    const C t = u[2] * u[2] * ej[2];
    ds[3] = C{-t.x, -t.y};  // Re r3: conj(r3) moves by dx
    ds[4] = C{-t.y, t.x};   // Im r3: conj(r3) moves by -i dy
  }
}

__device__ __forceinline__ void split_point_grad(double a, double b, double rho, double &sp, double &da, double &db,
                                                 double &drho) {
  const double absd = fabs(b - a);
  const double sg = b > a ? 1.0 : (b < a ? -1.0 : 0.0);
  if (0.5 * absd <= 2 * rho) {
    sp = a + 0.5 * absd;
    da = 1.0 - 0.5 * sg;
    db = 0.5 * sg;
    drho = 0.0;
  } else if (b > a) {
    sp = b - 2 * rho;
    da = 0.0;
    db = 1.0;
    drho = -2.0;
  } else {
    sp = b + 2 * rho;
    da = 0.0;
    db = 1.0;
    drho = 2.0;
  }
}

// The lens as the FP64 recomputation below needs it, passed by value so the
// caller's item stays in registers.
template <int NL>
struct NodeLens {
  cd r[NL];
  double eps[NL];
};

// 1 - |s/rho|^2 at one node in FP64, at the FP64 quadrature's node position
// d = hw t + mid (relative to the contour point), with the FP64 quadrature's
// arithmetic.  Where a node lies near a crossing of the limb, 1 - r^2 is a
// difference of O(|s/rho - uc|) terms that nearly cancel; its FP32 rounding
// (~1e-7 of those terms) then reaches the value itself, and dB/dr ~
// 1/sqrt(1 - r^2) amplifies it without bound (measured: a node 1.3e-8 inside
// the limb gave the wrong sign in FP32 and a per-point gradient off by 100 %).
template <int NL>
__device__ __noinline__ float limb_gap_fp64(NodeLens<NL> L, cd zc, cd w0, double rho, double d, int isQ) {
  const double inv_rho = 1.0 / rho;
  cd w = zc;
#pragma unroll
  for (int k = 0; k < NL; ++k) w = w - crecip(conj(zc) - conj(L.r[k])) * L.eps[k];
  const cd uc = (w - w0) * inv_rho;
  const double c1 = 1.0 - (uc.x * uc.x + uc.y * uc.y);
  const cd cdl = isQ ? mk(d, 0.0) : mk(0.0, -d);
  cd dl = isQ ? mk(d * inv_rho, 0.0) : mk(0.0, d * inv_rho);
#pragma unroll
  for (int k = 0; k < NL; ++k) {
    const cd D = conj(zc) - conj(L.r[k]);
    dl = dl + cdl * crecip(D + cdl) * crecip(D) * (L.eps[k] * inv_rho);
  }
  return (float)(c1 - 2.0 * (uc.x * dl.x + uc.y * dl.y) - (dl.x * dl.x + dl.y * dl.y));
}

// FP32 nodes recompute 1 - r^2 in FP64 where |1 - r^2| < X1_COND (|dl| + |dl|^2),
// i.e. where its FP32 rounding (bounded by ~8 eps32 (|dl| + |dl|^2)) exceeds
// 1e-2 of it: ~3e-5 of the nodes on the gradient workload's worst evaluations
// (CPU emulation of this arithmetic on the reference's contours).  Measured on
// that workload: thresholds 3x and 10x higher left every per-point gradient
// difference to FP64 the same to three digits and cost 1.6 % and 5 % more time.
constexpr float X1_COND = 1e2f * 8.0f * 5.9604645e-8f;

template <int NL, typename R, typename C>
__device__ void ld_pq_grad(const EsParams &P, const EsItem &It, cd zc, cd z0, PQGrad<GradDirs<NL>::NK> &g,
                           const float (*glf)[4][GL_MAX]) {
  constexpr int NK = GradDirs<NL>::NK, NLD = GradDirs<NL>::NLENS;
  // The direct parameter terms Ck (rho, u1, w0, lens) sum node values that no
  // image tangent multiplies later; the double-word nodes, which exist for the
  // terms the tangents amplify (the value and the position derivatives), keep
  // them in FP32.
  using CkT = typename std::conditional<std::is_same<R, dw>::value, float, R>::type;
  // shifted lens equation around the contour point
  const double rho = It.rho, inv_rho = 1.0 / rho;
  // D_j = conj(zc) - conj(r_j) and 1 / D_j, which lens_eq(zc) = zc - sum_j
  // eps_j / D_j uses too (the same operations in the same order as lens_eq)
  C Dj[NL], iDj[NL];
  R ej[NL];
  cd lez = zc;
#pragma unroll
  for (int k = 0; k < NL; ++k) {
    cd d = conj(zc) - conj(It.L.r[k]);
    cd id = crecip(d);
    lez = lez - id * It.L.eps[k];
    Dj[k] = C{(R)d.x, (R)d.y};
    iDj[k] = C{(R)id.x, (R)id.y};
    ej[k] = (R)It.L.eps[k];
  }
  const cd uc64 = (lez - It.w0) * inv_rho;  // (lens_eq(zc) - w0) / rho
  C uc = C{(R)uc64.x, (R)uc64.y};
  const R irho = (R)inv_rho, u1 = (R)It.u1;
  const R c0 = (R)(3.0 / (3.0 - It.u1)), dc0 = (R)(3.0 / ((3.0 - It.u1) * (3.0 - It.u1)));
  // 1 - |s/rho|^2 = (1 - |uc|^2) - 2 Re(conj(uc) dl) - |dl|^2 with the first
  // term in FP64: dB/dr ~ 1/sqrt(1 - r^2) near the limb, so 1 - r^2 must carry
  // an error relative to itself, not the rounding of r.
  const R c1 = (R)(1.0 - (uc64.x * uc64.x + uc64.y * uc64.y));
#pragma unroll
  for (int isQ = 0; isQ < 2; ++isQ) {
    const double a = isQ ? z0.x : z0.y, b = isQ ? zc.x : zc.y;
    double sp, dsa, dsb, dsr;
    split_point_grad(a, b, rho, sp, dsa, dsb, dsr);
    // the two halves' sums: FP64 for the FP64 quadrature, FP32 for FP32 nodes
    // (the halves cancel by at most a factor 2: the reference's split point
    // a + |b - a| / 2 can lie beyond a when b < a)
    R val = 0, fixed = 0, kk[NK], dlo[2], dhi[2];
#pragma unroll
    for (int k = 0; k < NK; ++k) kk[k] = 0;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const double lo = half ? sp : a, hi = half ? b : sp;
      const R lo_r = (R)(lo - b), hi_r = (R)(hi - b);
      const R hw = (R)0.5 * (hi_r - lo_r), mid = (R)0.5 * (hi_r + lo_r);
      const int n = half ? P.n2 : P.n1;
      R A = 0, Bl = 0, Bh = 0, Cf = 0;
      CkT Ck[NK];
#pragma unroll
      for (int k = 0; k < NK; ++k) Ck[k] = 0;
      for (int j = 0; j < n; ++j) {
        R t, w;
        if constexpr (std::is_same<R, float>::value) {
          t = glf[half][0][j];
          w = glf[half][1][j];
        } else if constexpr (std::is_same<R, dw>::value) {
          t = dw(glf[half][0][j], glf[half][2][j]);
          w = dw(glf[half][1][j], glf[half][3][j]);
        } else {
          t = P.gl_x[half][j];
          w = P.gl_w[half][j];
        }
        const R d = hw * t + mid;
        const C cdl = isQ ? C{d, (R)0} : C{(R)0, -d};  // conj(delta)
        // s/rho = uc + delta/rho + sum eps conj(delta) / (D (D + conj(delta))) / rho
        C dl = isQ ? C{d * irho, (R)0} : C{(R)0, d * irho};
        C u[NL];
#pragma unroll
        for (int k = 0; k < NL; ++k) {
          if constexpr (std::is_same<R, float>::value)
            u[k] = crecip_fast(Dj[k] + cdl);
          else
            u[k] = crecip(Dj[k] + cdl);
          dl = dl + cdl * u[k] * iDj[k] * (ej[k] * irho);
        }
        const C srho = C{uc.x + dl.x, uc.y + dl.y};
        R x1 = c1 - (R)2 * (uc.x * dl.x + uc.y * dl.y) - (dl.x * dl.x + dl.y * dl.y);  // 1 - r^2
        if constexpr (std::is_same<R, float>::value) {
          const float dln = fabsf(dl.x) + fabsf(dl.y);
          if (fabsf(x1) < X1_COND * dln * (1.0f + dln)) {
            NodeLens<NL> nl;
#pragma unroll
            for (int k = 0; k < NL; ++k) {
              nl.r[k] = It.L.r[k];
              nl.eps[k] = It.L.eps[k];
            }
            const double d64 = fma(0.5 * ((hi - b) - (lo - b)), P.gl_x[half][j], 0.5 * ((hi - b) + (lo - b)));
            x1 = limb_gap_fp64<NL>(nl, zc, It.w0, rho, d64, isQ);
          }
        }
        // r = |s/rho| and its reciprocal; B(r) and dB/dr.  FP32 nodes take
        // the approximate reciprocal and rsqrt (a few ulp, inside the FP32
        // rounding the node values carry already) for the IEEE divisions and
        // square roots, as the forward's nodes do
        R r, ir, B, dB;
        if constexpr (std::is_same<R, float>::value) {
          const float n2 = norm2(srho);
          ir = n2 > 0.0f ? rsqrtf(n2) : 0.0f;
          r = n2 * ir;
          if (x1 >= 0.0f) {
            const float rs = x1 > 0.0f ? rsqrtf(x1) : 0.0f;
            B = 1.0f + x1 * rs;
            dB = -r * rs;
          } else {
            const float x = -x1 * ir * ir;  // 1 - 1/r^2
            const float rs = rsqrtf(x);
            B = 1.0f - x * rs;
            dB = -(ir * ir * ir) * rs;
          }
        } else {
          r = cabs(srho);
          ir = r > (R)0 ? (R)1 / r : (R)0;
          if (x1 >= (R)0) {
            const R sq = msqrt(x1);
            B = (R)1 + sq;
            dB = x1 > (R)0 ? -r / sq : (R)0;
          } else {
            const R r2 = r * r, x = -x1 / r2;  // 1 - 1/r^2
            const R sq = msqrt(x);
            B = (R)1 - sq;
            dB = -(R)1 / (r2 * r * sq);
          }
        }
        const R I = c0 * (u1 * B + (R)1 - (R)2 * u1);
        const R dIdr = c0 * u1 * dB;
        const R dIdu1 = dc0 * (u1 * B + (R)1 - (R)2 * u1) + c0 * (B - (R)2);
        // unit vector of s, and d r = Re(conj(shat) ds) / rho
        const C sh = C{srho.x * ir, srho.y * ir};
        C lam = u[0] * u[0] * ej[0];
#pragma unroll
        for (int k = 1; k < NL; ++k) lam = lam + u[k] * u[k] * ej[k];
        // d s / d x' = 1 + lam ; d s / d y' = i (1 - lam)
        const R drx = (sh.x * ((R)1 + lam.x) + sh.y * lam.y) * irho;
        const R dry = (sh.x * lam.y + sh.y * ((R)1 - lam.x)) * irho;
        const R dr_along = isQ ? drx : dry, dr_fixed = isQ ? dry : drx;
        const R Iy = dIdr * dr_along;
        const R wI = w * I;
        A += wI;
        Bl += w * Iy * (R)0.5 * ((R)1 - t);
        Bh += w * Iy * (R)0.5 * ((R)1 + t);
        Cf += w * dIdr * dr_fixed;
        if constexpr (std::is_same<R, dw>::value) {
          // the direct parameter terms from the high words, in FP32
          const float wd = w.hi * dIdr.hi, irf = irho.hi, shx = sh.x.hi, shy = sh.y.hi;
          cf uf[NL], dslf[NLD];
          float ejf[NL];
#pragma unroll
          for (int k = 0; k < NL; ++k) {
            uf[k] = cf{u[k].x.hi, u[k].y.hi};
            ejf[k] = ej[k].hi;
          }
          lens_shifts<NL, float, cf>(uf, ejf, dslf);
          Ck[GK_RHO] += wd * (-r.hi * irf);
          Ck[GK_U1] += w.hi * dIdu1.hi;
          Ck[GK_WX] += wd * (-shx * irf);
          Ck[GK_WY] += wd * (-shy * irf);
#pragma unroll
          for (int m = 0; m < NLD; ++m) Ck[GK_A + m] += wd * ((shx * dslf[m].x + shy * dslf[m].y) * irf);
        } else {
          C dsl[NLD];
          lens_shifts<NL, R, C>(u, ej, dsl);
          Ck[GK_RHO] += w * dIdr * (-r * irho);
          Ck[GK_U1] += w * dIdu1;
          Ck[GK_WX] += w * dIdr * (-sh.x * irho);
          Ck[GK_WY] += w * dIdr * (-sh.y * irho);
#pragma unroll
          for (int m = 0; m < NLD; ++m) Ck[GK_A + m] += w * dIdr * ((sh.x * dsl[m].x + sh.y * dsl[m].y) * irho);
        }
      }
      val += hw * A;
      fixed += hw * Cf;
#pragma unroll
      for (int k = 0; k < NK; ++k) kk[k] += hw * (R)Ck[k];
      dlo[half] = (R)-0.5 * A + hw * Bl;
      dhi[half] = (R)0.5 * A + hw * Bh;
    }
    const double dsp = (double)dhi[0] + (double)dlo[1];
    const double d_a = (double)dlo[0] + dsp * dsa, d_b = (double)dhi[1] + dsp * dsb;
    const double f = isQ ? 0.5 : -0.5;
    if (!isQ) {
      g.P = f * (double)val;
      g.Py = f * d_b;
      g.Pa = f * d_a;
      g.Px = f * (double)fixed;
#pragma unroll
      for (int k = 0; k < NK; ++k) g.Pk[k] = f * (double)kk[k];
      g.Pk[GK_RHO] += f * dsp * dsr;
    } else {
      g.Q = f * (double)val;
      g.Qx = f * d_b;
      g.Qa = f * d_a;
      g.Qy = f * (double)fixed;
#pragma unroll
      for (int k = 0; k < NK; ++k) g.Qk[k] = f * (double)kk[k];
      g.Qk[GK_RHO] += f * dsp * dsr;
    }
  }
}


// Tangents dz/dtheta of an image z of a limb point, for the parameter
// directions of GradDirs: from lens_eq(z) = w0 + rho e^{i th},
// dz = (g - lam conj(g)) / (1 - |lam|^2), lam = sum_j eps_j / (conj(z) - conj(r_j))^2,
// g = the source-plane shift the parameter produces at fixed z (w0 and rho
// move the source; the lens directions move the lens equation by -lens_shifts).
// e^{i th} = (lens_eq(z) - w0) / rho comes from the reciprocals computed here
// anyway (a few FP64 operations where sincos(th) takes tens; the image's
// residual, ~1e-15, puts it within ~1e-15 / rho of the limb's value).
template <int NL>
__device__ __forceinline__ void image_tangents(const EsItem &I, cd z, cd (&t)[GradDirs<NL>::NK]) {
  constexpr int NLD = GradDirs<NL>::NLENS;
  cd u[NL];
  double ej[NL];
#pragma unroll
  for (int k = 0; k < NL; ++k) {
    u[k] = crecip(conj(z) - conj(I.L.r[k]));
    ej[k] = I.L.eps[k];
  }
  cd lam = u[0] * u[0] * ej[0];
#pragma unroll
  for (int k = 1; k < NL; ++k) lam = lam + u[k] * u[k] * ej[k];
  const double iD = 1.0 / (1.0 - norm2(lam));
  cd e = z;
#pragma unroll
  for (int k = 0; k < NL; ++k) e = e - u[k] * ej[k];
  e = (e - I.w0) * (1.0 / I.rho);
  cd dsl[NLD];
  lens_shifts<NL, double, cd>(u, ej, dsl);
  cd g[4 + NLD] = {e, mk(0.0, 0.0), mk(1.0, 0.0), mk(0.0, 1.0)};
#pragma unroll
  for (int m = 0; m < NLD; ++m) g[4 + m] = mk(-dsl[m].x, -dsl[m].y);
#pragma unroll
  for (int k = 0; k < 4 + NLD; ++k) t[k] = (g[k] - lam * conj(g[k])) * iD;
}

// Backward pass of one extended-source evaluation (binary lenses): the
// contours of the forward pass are recomputed, never stored between passes.
// T = sum_c parity_c I_c, mu = |T| / (pi rho^2).
template <int NL, int PREC>
__device__ void es_backward(const EsParams &P, EsSmem<NL * NL + 1> &S, const EsItem &I, int ncont, int ntot,
                            const int *cstart, const int *cpar, const cd *centroid,
                            double (*contour_acc)[MAX_CLOSED + N_CONTOURS], double (*cgr)[2],
                            double (*cgr_w)[MAX_CLOSED + N_CONTOURS][2], double (*pgr_w)[NK_MAX], double *tot_sh,
                            int64_t pi, double *mag, const float (*glf)[4][GL_MAX]) {
  constexpr int NK = GradDirs<NL>::NK;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    double tot = 0.0;
    for (int c = 0; c < ncont; ++c) {
      double s = 0.0;
      for (int w = 0; w < ES_WARPS; ++w) s += contour_acc[w][c];
      tot += s * cpar[c];
    }
    *tot_sh = tot;
  }
  for (int i = tid; i < ntot; i += ES_THREADS) S.GG[i] = mk(0, 0);
  __syncthreads();
  // pass 2: node-level derivatives, trapezoid weights, centroids, direct terms.
  // Sums over points run in a fixed order (per-thread partials, shuffle trees,
  // per-warp slots summed in warp order): two identical calls give identical bits.
  double acc[NK];
#pragma unroll
  for (int k = 0; k < NK; ++k) acc[k] = 0.0;
  {
    int c = 0;
    for (int base = warp * 32; base < ntot; base += ES_THREADS) {  // warp-uniform trip count
      const int i = base + lane;
      double cg0 = 0.0, cg1 = 0.0;  // this point's d T / d(x0_c, y0_c)
      int key = -1;
      if (i < ntot) {
        while (i >= cstart[c + 1]) ++c;
        key = c;
        const int b = cstart[c], e = min(cstart[c + 1], ntot);
        const double pc = cpar[c];
        const int ip = i > b ? i - 1 : i, in = i + 1 < e ? i + 1 : i;
        const cd zc = S.Z[S.CP[i]], zp = S.Z[S.CP[ip]], zn = S.Z[S.CP[in]];
        if (P.ld) {
          const double wx = 0.5 * (zn.x - zp.x), wy = 0.5 * (zn.y - zp.y);
          // wx_i = (x_in - x_ip)/2, wy_i = (y_in - y_ip)/2, so P_i wx_i + Q_i wy_i
          // contributes P_i (t_in - t_ip).x / 2 + Q_i (t_in - t_ip).y / 2 per
          // parameter.  Summed by parts against the FP64 image tangents rather than
          // scattered into the neighbours' position adjoints, where it would become
          // (P_ip - P_in) / 2: a difference of nearly equal quadrature values that
          // amplifies their rounding (FP32 nodes) by |P| / |dP| ~ 1e4.
          // Near a critical curve the tangents grow like 1/|det J| and the
          // pointwise contributions cancel in the sum; there the FP32 node values
          // (relative error ~1e-7) would be amplified, so such points run the
          // quadrature in FP64 (double-word under mixed precision).  Only the
          // differences t_in - t_ip stay live across the quadrature.
          double amp2 = 0.0;
          cd dt[NK];
          {
            cd t[NK];
            image_tangents<NL>(I, zn, t);
  #pragma unroll
            for (int k = 0; k < NK; ++k) {
              amp2 = fmax(amp2, norm2(t[k]));
              dt[k] = t[k];
            }
            image_tangents<NL>(I, zp, t);
  #pragma unroll
            for (int k = 0; k < NK; ++k) {
              amp2 = fmax(amp2, norm2(t[k]));
              dt[k] = mk(dt[k].x - t[k].x, dt[k].y - t[k].y);
            }
            image_tangents<NL>(I, zc, t);
  #pragma unroll
            for (int k = 0; k < NK; ++k) amp2 = fmax(amp2, norm2(t[k]));
          }
          PQGrad<NK> g;
          if (PREC == MIXED && amp2 <= P.grad_amp2)
            ld_pq_grad<NL, float, cf>(P, I, zc, centroid[c], g, glf);
          else
            ld_pq_grad<NL, typename std::conditional<PREC == MIXED, dw, double>::type,
                       typename std::conditional<PREC == MIXED, cdw, cd>::type>(P, I, zc, centroid[c], g, glf);
          const cd pq = mk(g.P, g.Q);
          atomicAdd(&S.GG[i].x, pc * (wx * g.Px + wy * g.Qx));
          atomicAdd(&S.GG[i].y, pc * (wx * g.Py + wy * g.Qy));
  #pragma unroll
          for (int k = 0; k < NK; ++k)
            acc[k] += 0.5 * pc * (pq.x * dt[k].x + pq.y * dt[k].y);
          cg1 = pc * wx * g.Pa;
          cg0 = pc * wy * g.Qa;
  #pragma unroll
          for (int k = 0; k < NK; ++k) acc[k] += pc * (wx * g.Pk[k] + wy * g.Qk[k]);
        } else if (i + 1 < e) {
          // pair (i, i+1): 1/4 [(x_i + x_{i+1})(y_{i+1} - y_i) - (y_i + y_{i+1})(x_{i+1} - x_i)];
          // each GG entry receives exactly two addends onto zero, an order-free sum
          const cd a = zc, q = zn;
          atomicAdd(&S.GG[i].x, pc * 0.5 * q.y);
          atomicAdd(&S.GG[i].y, -pc * 0.5 * q.x);
          atomicAdd(&S.GG[i + 1].x, -pc * 0.5 * a.y);
          atomicAdd(&S.GG[i + 1].y, pc * 0.5 * a.x);
        }
      }
      if (P.ld) {
        warp_run_add(key, cg0, &cgr_w[warp][0][0], 2);
        warp_run_add(key, cg1, &cgr_w[warp][0][1], 2);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < NK; ++k) {
    double v = acc[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) pgr_w[warp][k] += v;
    acc[k] = 0.0;
  }
  __syncthreads();
  for (int q = tid; q < 2 * ncont; q += ES_THREADS) {  // per-contour sums in warp order
    double v = 0.0;
    for (int w = 0; w < ES_WARPS; ++w) v += cgr_w[w][q >> 1][q & 1];
    cgr[q >> 1][q & 1] = v;
  }
  __syncthreads();
  // pass 3: every contour point's image through the lens equation:
  // dz + lam conj(dz) = g (image_tangents), lam = sum eps/(conj z - conj r)^2
  {
    int c = 0;
    for (int i = tid; i < ntot; i += ES_THREADS) {
      while (i >= cstart[c + 1]) ++c;
      const int b = cstart[c], e = min(cstart[c + 1], ntot);
      cd G = S.GG[i];
      if (P.ld) {
        const double inv_n = 1.0 / (double)(e - b);
        G = G + mk(cgr[c][0] * inv_n, cgr[c][1] * inv_n);
      }
      const uint32_t cp = S.CP[i];
      cd t[NK];
      image_tangents<NL>(I, S.Z[cp], t);
#pragma unroll
      for (int k = 0; k < NK; ++k) acc[k] += G.x * t[k].x + G.y * t[k].y;
    }
  }
#pragma unroll
  for (int k = 0; k < NK; ++k) {
    double v = acc[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) pgr_w[warp][k] += v;
  }
  __syncthreads();
  if (tid == 0) {
    const double tot = *tot_sh, rho = I.rho;
    const double mu = fabs(tot) / (3.14159265358979323846 * rho * rho);
    const double sT = (tot > 0 ? 1.0 : (tot < 0 ? -1.0 : 0.0)) / (3.14159265358979323846 * rho * rho);
    double d[NK];
    for (int k = 0; k < NK; ++k) {
      double v = 0.0;
      for (int w = 0; w < ES_WARPS; ++w) v += pgr_w[w][k];
      d[k] = sT * v;
    }
    d[GK_RHO] -= 2.0 * mu / rho;
    // (a, e1, x_cm) -> (s, q): a = s/2, e1 = 1/(1+q), x_cm = a(1-q)/(1+q);
    // triple (point_source.py:1807-1817): e1 = q/(1+q+q3), e2 = q e1, r3 = R e^{i psi}
    const double q = I.q, a = 0.5 * I.s, opq = 1.0 + q;
    const double ds = 0.5 * d[GK_A] + d[GK_WX] * (1.0 - q) / (2.0 * opq);
    double dq, dq3 = 0.0, dr3 = 0.0, dpsi = 0.0;
    if constexpr (NL == 2) {
      dq = -d[GK_E1] / (opq * opq) - d[GK_WX] * 2.0 * a / (opq * opq);
    } else {
      const double den = 1.0 + q + I.q3, e1 = q / den;
      const double e1_q = (1.0 + I.q3) / (den * den), e1_q3 = -q / (den * den);
      dq = d[GK_E1] * e1_q + d[GK_E2] * (e1 + q * e1_q) - d[GK_WX] * 2.0 * a / (opq * opq);
      double sp, cp;
      sincos(I.psi, &sp, &cp);
      dq3 = d[GK_E1] * e1_q3 + d[GK_E2] * q * e1_q3;
      dr3 = d[GK_R3X] * cp + d[GK_R3Y] * sp;
      dpsi = I.r3 * (-d[GK_R3X] * sp + d[GK_R3Y] * cp);
      if (P.gout && I.curve < 0) {
        double *gp = P.gout + pi * 9;
        gp[6] = dq3;
        gp[7] = dr3;
        gp[8] = dpsi;
      }
    }
    mag[pi] = mu;
    if (I.curve >= 0 && P.grow) {
      double u0, alpha, tE;
      if constexpr (NL == 2) {
        const CurveDev cv = P.curves[I.curve];
        u0 = cv.u0, alpha = cv.alpha, tE = cv.tE;
      } else {
        const CurveDev3 cv = P.curves3[I.curve];
        u0 = cv.u0, alpha = cv.alpha, tE = cv.tE;
      }
      const double ct = P.cot ? P.cot[pi] : 1.0;
      double sa, ca;
      sincos(alpha, &sa, &ca);
      const double tau = I.tau;
      // w = (u0 cos a + tau sin a) + i (-u0 sin a + tau cos a), tau = (t - t0)/tE
      const double du0 = d[GK_WX] * ca - d[GK_WY] * sa;
      const double dal = d[GK_WX] * (-u0 * sa + tau * ca) + d[GK_WY] * (-u0 * ca - tau * sa);
      const double dt0 = -(d[GK_WX] * sa + d[GK_WY] * ca) / tE;
      const double dtE = -tau * (d[GK_WX] * sa + d[GK_WY] * ca) / tE;
      // this point's cotangent-weighted row in the curve's parameter order;
      // curve_grad_reduce_kernel sums the rows of each curve in a fixed order
      if constexpr (NL == 2) {
        double *gp = P.grow + pi * 8;
        gp[0] = ct * ds;
        gp[1] = ct * dq;
        gp[2] = ct * d[GK_RHO];
        gp[3] = ct * d[GK_U1];
        gp[4] = ct * du0;
        gp[5] = ct * dal;
        gp[6] = ct * dt0;
        gp[7] = ct * dtE;
      } else {  // (s, q, q3, r3, psi, rho, u1, u0, alpha, t0, tE)
        double *gp = P.grow + pi * 11;
        gp[0] = ct * ds;
        gp[1] = ct * dq;
        gp[2] = ct * dq3;
        gp[3] = ct * dr3;
        gp[4] = ct * dpsi;
        gp[5] = ct * d[GK_RHO];
        gp[6] = ct * d[GK_U1];
        gp[7] = ct * du0;
        gp[8] = ct * dal;
        gp[9] = ct * dt0;
        gp[10] = ct * dtE;
      }
    } else if (P.gout) {
      double *gp = P.gout + pi * (NL == 2 ? 6 : 9);
      gp[0] = ds;
      gp[1] = dq;
      gp[2] = d[GK_RHO];
      gp[3] = d[GK_U1];
      gp[4] = d[GK_WX];
      gp[5] = d[GK_WY];
    }
  }
}

// Source, lens and limb-darkening parameters of point pi: a batched light
// curve's point (curve by bisection of offsets, rectilinear trajectory), or a
// source centre of a single lens.
__device__ __forceinline__ EsItem make_item(const EsParams &P, const cd *w0s, int64_t pi) {
  EsItem it;
  if (P.curves3) {  // triple-lens light curves
    int64_t lo = 0, hi = P.ncurves - 1;
    while (lo < hi) {
      const int64_t mid = (lo + hi + 1) >> 1;
      if (P.offsets[mid] <= pi) lo = mid; else hi = mid - 1;
    }
    const CurveDev3 cv = P.curves3[lo];
    it.L = make_lens(3, cv.s, cv.q, cv.q3, cv.r3, cv.psi);
    it.rho = cv.rho;
    it.u1 = P.ld ? cv.u1 : 0.0;
    const double tau = (P.times[pi] - cv.t0) / cv.tE;
    double sa, ca;
    sincos(cv.alpha, &sa, &ca);
    it.w0 = mk(cv.u0 * ca + tau * sa + it.L.x_cm, -cv.u0 * sa + tau * ca);
    it.s = cv.s;
    it.q = cv.q;
    it.q3 = cv.q3;
    it.r3 = cv.r3;
    it.psi = cv.psi;
    it.curve = lo;
    it.tau = tau;
  } else if (P.curves) {
    int64_t lo = 0, hi = P.ncurves - 1;
    while (lo < hi) {
      const int64_t mid = (lo + hi + 1) >> 1;
      if (P.offsets[mid] <= pi) lo = mid; else hi = mid - 1;
    }
    const CurveDev cv = P.curves[lo];
    it.L = make_lens(2, cv.s, cv.q, 0.0, 0.0, 0.0);
    it.rho = cv.rho;
    it.u1 = P.ld ? cv.u1 : 0.0;
    const double tau = (P.times[pi] - cv.t0) / cv.tE;
    double sa, ca;
    sincos(cv.alpha, &sa, &ca);
    it.w0 = mk(cv.u0 * ca + tau * sa + it.L.x_cm, -cv.u0 * sa + tau * ca);
    it.s = cv.s;
    it.q = cv.q;
    it.q3 = it.r3 = it.psi = 0.0;
    it.curve = lo;
    it.tau = tau;
  } else {
    it.L = P.L;
    it.rho = P.rho;
    it.u1 = P.u1;
    const cd w = w0s[pi];
    it.w0 = mk(w.x + P.L.x_cm, w.y);
    it.s = P.s_user;
    it.q = P.q_user;
    it.q3 = P.q3_user;
    it.r3 = P.r3_user;
    it.psi = P.psi_user;
    it.curve = -1;
    it.tau = 0.0;
  }
  return it;
}

// Limb angle of initial point k: jnp.linspace(-pi, pi, n0 - 1, endpoint=False)
// then pi - 1e-8, rounded as NumPy does.
__device__ __forceinline__ double limb_theta(int k, int n0) {
  const double step = 6.283185307179586 / (double)(n0 - 1);
  return (k < n0 - 1) ? __dadd_rn(__dmul_rn((double)k, step), -3.141592653589793) : 3.141592653589793 - 1e-8;
}

// Row order of the first limb point for every item of a launch, ahead of the
// contour kernel (which then reads perm0[item] instead of solving): one group
// of DEG lanes per item (one lane per root), 32 / DEG groups per warp (6 of 5
// lanes for binary lenses, 3 of 10 for triple), so each FP64 instruction of
// the reference's cold-start iteration serves that many items.  Lane 0 of a
// group first repeats the contour kernel's fast solve of that point (same
// polynomial, same deterministic solver), whose roots are the raw rows to
// order.  Items are enumerated exactly as the contour kernel takes them.
constexpr int FO_THREADS = 128;
template <int NL, int PREC, bool EARLY>
__global__ void __launch_bounds__(FO_THREADS) es_first_order_kernel(const EsParams P, const cd *__restrict__ w0s,
                                                                   const int64_t *__restrict__ index,
                                                                   const uint8_t *__restrict__ route,
                                                                   int64_t npoints, uint64_t *__restrict__ perm0) {
  constexpr int DEG = NL * NL + 1, G = DEG, GW = 32 / G, NG = GW * (FO_THREADS / 32);
  __shared__ cd zs[NG][DEG];
  // the contour kernel may start its limb sampling now; it waits for this
  // grid's completion (griddepcontrol.wait) before it reads perm0
  asm volatile("griddepcontrol.launch_dependents;");
  const int lane = threadIdx.x & 31, gw = lane / G;
  if (gw >= GW) return;  // the lanes past the warp's last whole group
  const int g = (threadIdx.x >> 5) * GW + gw, r = lane - gw * G;
  const unsigned gmask = refea::gmask_of<G>();
  const int64_t nitems = P.qhead ? *P.qcount : npoints;
  for (int64_t it = (int64_t)blockIdx.x * NG + g; it < nitems; it += (int64_t)gridDim.x * NG) {
    const int64_t pi = P.qhead ? P.qlist[it] : (index ? index[it] : it);
    if (route && route[pi] == 0) continue;  // uniform over the group
    const EsItem I = make_item(P, w0s, pi);
    const double th = limb_theta(0, P.n0);
    if (r == 0) {
      cd z[DEG];
      uint16_t mkb, pp, zp;
      uint32_t flags = 0;
      solve_limb_point<NL, PREC, EARLY>(P, I, th, z, nullptr, mkb, pp, zp, flags);
#pragma unroll
      for (int i = 0; i < DEG; ++i) zs[g][i] = z[i];
    }
    __syncwarp(gmask);
    int its;
    const uint64_t o = first_point_order_group<NL, G>(P, I, th, zs[g], its);
    if (r == 0) perm0[it] = o;
    __syncwarp(gmask);
  }
}

template <int NL, int PREC, bool GRAD = false>
__global__ void __launch_bounds__(ES_MAX_THREADS, NL == 2 ? 2 : 1) es_kernel(const EsParams P, const cd *__restrict__ w0s,
                                                        const int64_t *__restrict__ index,
                                                        const uint8_t *__restrict__ route, int64_t npoints,
                                                        double *__restrict__ mag, uint32_t *__restrict__ status) {
  constexpr int DEG = NL * NL + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int warp_tot[ES_MAX_WARPS];
  __shared__ double contour_acc[ES_MAX_WARPS][MAX_CLOSED + N_CONTOURS];
  __shared__ cd centroid[MAX_CLOSED + N_CONTOURS];
  __shared__ int cstart[MAX_CLOSED + N_CONTOURS + 1];
  __shared__ int cpar[MAX_CLOSED + N_CONTOURS];
  __shared__ uint32_t sflags;
  __shared__ int nsel_sh;
  __shared__ int nlist_sh;
  __shared__ int dbg_ref[7];  // diagnostics: first-point iterations; A: solves, iterations; B: solves,
                             // iterations; refinement FP32-stage iterations, refinement points
  __shared__ long long dbg_b[ES_DBG_SUB];  // diagnostics: refinement clocks (gaps+rank+scan, FP32 stages or
                                           // whole solves, polish + filter, per-point labelling, faithful, insertion)
  __shared__ long long dbg_arr[ES_MAX_WARPS];  // diagnostics: each warp's clock on reaching a barrier
  __shared__ long long clk[8];
  __shared__ int64_t item_sh, iord_sh;  // point index, item ordinal
  __shared__ EsItem item;
  __shared__ double cgr[MAX_CLOSED + N_CONTOURS][2];  // adjoint: dT/dx0_c, dT/dy0_c
  // adjoint partial sums per warp (summed in warp order): dT/d(x0_c, y0_c) and
  // the direct dT/d(rho, u1, w0x, w0y, a, e1)
  __shared__ double cgr_w[GRAD ? ES_MAX_WARPS : 1][MAX_CLOSED + N_CONTOURS][2];
  __shared__ double pgr_w[GRAD ? ES_MAX_WARPS : 1][NK_MAX];
  __shared__ double tot_sh;
  // FP32 Gauss-Legendre tables [half][nodes | weights | their low words][j]:
  // the FP32 nodes use the first two, the adjoint's double-word quadrature all four
  __shared__ float glf[2][4][GL_MAX];
  for (int i = threadIdx.x; i < 2 * GL_MAX; i += ES_THREADS) {
    const int h = i / GL_MAX, j = i % GL_MAX;
    const dw x(P.gl_x[h][j]), w(P.gl_w[h][j]);
    glf[h][0][j] = x.hi;
    glf[h][1][j] = w.hi;
    glf[h][2][j] = x.lo;
    glf[h][3][j] = w.lo;
  }
  const int Lcap = P.Lcap;
  EsSmem<DEG> S;
  {
    // Z, TH and CP stay live through the integrals and the adjoint; everything
    // after them is dead once the contour point lists exist, so the adjoint's
    // per-point accumulators GG reuse that region when it is large enough.
    unsigned char *p = smem_raw;
    S.Z = reinterpret_cast<cd *>(p);
    p += sizeof(cd) * (size_t)Lcap * DEG;
    S.TH = reinterpret_cast<double *>(p);
    p += sizeof(double) * Lcap;
    S.CP = reinterpret_cast<uint32_t *>(p);
    p += sizeof(uint32_t) * (size_t)P.CPcap;
    p = smem_raw + (((size_t)(p - smem_raw) + 15) / 16 * 16);
    unsigned char *const dead = p;
    S.KEY = reinterpret_cast<double *>(p);
    p += sizeof(double) * Lcap;
    S.PERM = reinterpret_cast<uint64_t *>(p);
    p += sizeof(uint64_t) * Lcap;
    S.BMAP = reinterpret_cast<uint64_t *>(p);
    p += sizeof(uint64_t) * Lcap;
    S.USED = reinterpret_cast<uint64_t *>(p);
    p += sizeof(uint64_t) * Lcap;
    S.CAND = reinterpret_cast<uint64_t *>(p);
    p += sizeof(uint64_t) * (size_t)Lcap * DEG;
    S.M = reinterpret_cast<MergeState *>(p);
    p += (sizeof(MergeState) + 15) / 16 * 16;
    S.SCAN = reinterpret_cast<int *>(p);
    p += sizeof(int) * (Lcap + 1);
    S.MK = reinterpret_cast<uint16_t *>(p);
    p += sizeof(uint16_t) * Lcap;
    S.PP = reinterpret_cast<uint16_t *>(p);
    p += sizeof(uint16_t) * Lcap;
    S.ZP = reinterpret_cast<uint16_t *>(p);
    p += sizeof(uint16_t) * Lcap;
    S.ORD = reinterpret_cast<uint16_t *>(p);
    p += sizeof(uint16_t) * Lcap;
    S.ORD2 = reinterpret_cast<uint16_t *>(p);
    p += sizeof(uint16_t) * Lcap;
    p = smem_raw + (((size_t)(p - smem_raw) + 15) / 16 * 16);
    S.GG = ((size_t)(p - dead) >= sizeof(cd) * (size_t)P.CPcap) ? reinterpret_cast<cd *>(dead)
                                                                  : reinterpret_cast<cd *>(p);
  }
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  // Items: static round-robin over [0, npoints), or a persistent device queue
  // (P.qhead) of *P.qcount point indices P.qlist taken P.qchunk at a time.
  int64_t chunk_next = 0, chunk_end = 0, static_next = blockIdx.x;
  for (;;) {
    if (tid == 0) {
      int64_t it;
      if (P.qhead) {
        if (chunk_next >= chunk_end) {
          chunk_next = (int64_t)atomicAdd(P.qhead, (unsigned long long)P.qchunk);
          chunk_end = chunk_next + P.qchunk;
        }
        it = chunk_next++;
        item_sh = it < *P.qcount ? P.qlist[it] : -1;
        iord_sh = it;
      } else {
        it = static_next;
        static_next += gridDim.x;
        item_sh = it < npoints ? (index ? index[it] : it) : -1;
        iord_sh = it;
      }
    }
    __syncthreads();
    const int64_t pi = item_sh;
    if (pi < 0) break;
    if (route && route[pi] == 0) {  // hexadecapole accepted (CTA-uniform)
      __syncthreads();
      continue;
    }
    if (tid == 0) {
      item = make_item(P, w0s, pi);
      sflags = 0;
    }
    uint32_t flags = 0;
    __syncthreads();
    const EsItem &I = item;
    if (!isfinite(I.w0.x) || !isfinite(I.w0.y)) {  // a non-finite source centre (CTA-uniform): not evaluated
      if (tid == 0) {
        const double nan = __longlong_as_double(0x7ff8000000000000ll);
        mag[pi] = nan;
        if (status) status[pi] = route ? (status[pi] | CGB_ST_INVALID) : CGB_ST_INVALID;
        if (GRAD && P.gout)
          for (int k = 0; k < (NL == 2 ? 6 : 9); ++k) P.gout[pi * (NL == 2 ? 6 : 9) + k] = nan;
      }
      __syncthreads();
      continue;
    }
    if (P.dbg && tid == 0) {
      clk[0] = clock64();
      for (int c = 0; c < 7; ++c) dbg_ref[c] = 0;
      for (int c = 0; c < ES_DBG_SUB; ++c) dbg_b[c] = 0;
    }

    // ---- A: initial limb sampling (extended_source.py:100-107) ----
    const int n0 = P.n0;
    for (int k = tid; k < n0; k += ES_THREADS) {
      const double th = limb_theta(k, n0);
      S.TH[k] = th;
      S.ORD[k] = (uint16_t)k;
      solve_limb_point<NL, PREC, !GRAD>(P, I, th, S.Z + (size_t)k * DEG, nullptr, S.MK[k], S.PP[k], S.ZP[k], flags);
    }
    if (P.dbg && lane == 0) dbg_arr[warp] = clock64();
    __syncthreads();
    long long ta = 0;  // diagnostics: end of the previous initial-sampling sub-phase (thread 0)
    auto arrival_max = [&]() {
      long long m = dbg_arr[0];
      for (int q = 1; q < ES_WARPS; ++q) m = max(m, dbg_arr[q]);
      return m;
    };
    if (P.dbg && tid == 0) {
      ta = arrival_max();
      dbg_b[6] += ta - clk[0];
    }
    if (P.dbg) __syncthreads();
    // Row order of the reference's sequential warm-start chain, emulated in
    // parallel: clear steps take the nearest-root map; ambiguous steps rerun the
    // reference's warm start from the predecessor in the current chain order,
    // and the chain is recomposed until no ambiguous map moves.
    constexpr int RG = RefGroup<DEG>::G;
    if (P.nearest) {
      if (tid == 0) {
        uint64_t ident = 0;
        for (int t = 0; t < DEG; ++t) ident = perm_set(ident, t, t);
        S.PERM[0] = ident;
      }
    } else if (P.perm0) {  // ordered ahead of this kernel (es_first_order_kernel)
      if (tid == 0) {
        asm volatile("griddepcontrol.wait;" ::: "memory");  // that grid complete (at once when launched after it)
        S.PERM[0] = P.perm0[iord_sh];
      }
    } else if (tid < RG) {
      int its;
      const uint64_t o = first_point_order_group<NL>(P, I, S.TH[0], S.Z, its);
      if (tid == 0) {
        S.PERM[0] = o;
        if (P.dbg) dbg_ref[0] += its;
      }
    }
    for (int k = 1 + tid; k < n0; k += ES_THREADS) {
      bool amb;
      S.BMAP[k] = step_map<DEG>(S.Z + (size_t)(k - 1) * DEG, S.Z + (size_t)k * DEG, amb);
      S.USED[k] = (amb && !P.nearest) ? ~0ull : 0ull;  // 0: map final (clear step, or nearest labelling)
    }
    if (P.dbg && lane == 0) dbg_arr[warp] = clock64();
    __syncthreads();
    if (P.dbg && tid == 0) {
      const long long t = arrival_max();
      dbg_b[7] += t - ta;
      ta = t;
    }
    if (P.dbg) __syncthreads();
    for (int round = 0; round < 12; ++round) {
      if (tid == 0) {
        uint64_t ord = S.PERM[0];
        for (int k = 1; k < n0; ++k) {
          uint64_t b = S.BMAP[k], nw = 0;
          for (int t = 0; t < DEG; ++t) nw = perm_set(nw, t, perm_get(b, perm_get(ord, t)));
          S.PERM[k] = nw;
          ord = nw;
        }
        nsel_sh = 0;
        nlist_sh = 0;
      }
      __syncthreads();
      if (round == 11) {
        if (tid == 0) atomicOr(&sflags, CGB_ST_MERGE);
        break;
      }
      // steps whose map must be (re)computed from the current chain order
      for (int k = 1 + tid; k < n0; k += ES_THREADS) {
        const uint64_t prev = S.PERM[k - 1], used = S.USED[k];
        if (used == 0ull || used == prev) continue;
        S.SCAN[atomicAdd(&nlist_sh, 1)] = k;
      }
      __syncthreads();
      for (int e = tid / RG; e < nlist_sh; e += ES_THREADS / RG) {
        const int k = S.SCAN[e];
        const uint64_t prev = S.PERM[k - 1];
        int its;
        const uint64_t nb = warm_map_ref_group<NL>(P, I, S.TH[k], S.Z + (size_t)(k - 1) * DEG, prev,
                                                   S.Z + (size_t)k * DEG, false, its);
        if ((tid & (RG - 1)) == 0) {
          if (P.dbg) {
            atomicAdd(&dbg_ref[1], 1);
            atomicAdd(&dbg_ref[2], its);
          }
          if (nb != S.BMAP[k]) {
            S.BMAP[k] = nb;
            nsel_sh = 1;
          }
          S.USED[k] = prev;
        }
      }
      __syncthreads();
      const bool again = nsel_sh != 0;
      __syncthreads();
      if (!again) break;
    }
    for (int k = tid; k < n0; k += ES_THREADS)
      apply_rows<DEG>(S.Z + (size_t)k * DEG, S.MK[k], S.PP[k], S.ZP[k], S.PERM[k]);
    if (P.dbg && lane == 0) dbg_arr[warp] = clock64();
    __syncthreads();
    if (P.dbg && tid == 0) dbg_b[8] += arrival_max() - ta;
    if (P.dbg) __syncthreads();
    if (P.dbg && tid == 0) clk[1] = clock64();

    // ---- B: refinement rounds (extended_source.py:109-135) ----
    // The intervals are ranked (larger length first, ties: larger limb position
    // first) once, by a sort of the initial ones; a round then takes the head of
    // that list, and only the intervals next to its new points are sorted and
    // merged into the rest, whose order a round does not change (their
    // positions shift by the number of new points before them).  Lengths are
    // >= +0, so their IEEE bit patterns order as integers.  Storage in the
    // candidate lists' region, unused until the chained matching: the ranked
    // list (length bits, limb position), the selected interval of each new
    // point, then scratch: the initial sort's keys, the new points' solver
    // scratch, or the new intervals and the merged list.
    long long *SLV = reinterpret_cast<long long *>(S.CAND);                      // [Lcap]
    uint16_t *SLP = reinterpret_cast<uint16_t *>(SLV + Lcap);                     // [Lcap]
    int *NEWK = reinterpret_cast<int *>(S.CAND) + ((size_t)Lcap * 10 + 3) / 4;   // [n_add]
    unsigned char *rtmp = reinterpret_cast<unsigned char *>(S.CAND) +
                          (((size_t)Lcap * 10 + 4 + (size_t)P.n_add * 4 + 15) & ~(size_t)15);
    {
      const int m0 = n0 - 1;
      int nsort = 1;
      while (nsort < m0) nsort <<= 1;
      long long *SV = reinterpret_cast<long long *>(rtmp);
      uint16_t *SI = reinterpret_cast<uint16_t *>(SV + nsort);
      for (int k = tid; k < nsort; k += ES_THREADS) {
        SV[k] = k < m0 ? __double_as_longlong(interval_len<DEG>(S, S.ORD[k], S.ORD[k + 1])) : -1ll;
        SI[k] = (uint16_t)(k < m0 ? k : 0);
      }
      __syncthreads();
      bitonic_sort_desc(SV, SI, nsort);
      for (int k = tid; k < m0; k += ES_THREADS) {
        SLV[k] = SV[k];
        SLP[k] = SI[k];
      }
    }
    int Lcur = n0;
    long long tb = 0;
    for (int round = 0; round < P.niter; ++round) {
      if (P.dbg && tid == 0 && round == 0) tb = clock64();
      const int ngap = Lcur - 1;
      for (int k = tid; k <= ngap; k += ES_THREADS) S.SCAN[k] = 0;
      if (tid == 0) nlist_sh = 0;
      __syncthreads();  // the ranked list of the previous round complete
      for (int r = tid; r < P.n_add && r < ngap; r += ES_THREADS) S.SCAN[SLP[r]] = 1;
      __syncthreads();
      // positions of the selected gaps -> compact list in SCAN (exclusive scan)
      for (int k = tid; k <= ngap; k += ES_THREADS) S.KEY[k] = (double)S.SCAN[k];  // keep flags
      __syncthreads();
      if (P.dbg && lane == 0) dbg_arr[warp] = clock64();
      int nsel = block_exclusive_scan(S.SCAN, ngap + 1, warp_tot);  // synchronises the block
      for (int k = tid; k < ngap; k += ES_THREADS)
        if (S.KEY[k] != 0.0) NEWK[S.SCAN[k]] = k;
      __syncthreads();
      // each sub-phase ends when its last warp reaches the closing barrier
      auto last_arrival = [&]() {
        long long m = dbg_arr[0];
        for (int q = 1; q < ES_WARPS; ++q) m = max(m, dbg_arr[q]);
        return m;
      };
      if (P.dbg && tid == 0) {
        const long long t = last_arrival();
        dbg_b[0] += t - tb;
        tb = t;
      }
      if (P.dbg) __syncthreads();  // keep the arrival clocks until read
      // new slots: selected gap k -> slot Lcur + SCAN[k]
      if (PREC == MIXED) {
        // One new point per thread leaves a single warp doing the FP64 polish
        // and image filter of every root in turn, which made these solves the
        // longest path of the refinement; here the FP32 stages run per point,
        // then one lane per (point, root) polishes and filters, then one thread
        // per point checks the root set and labels it.  Scratch lives where the
        // ranking's sort keys were.
        cd *pco = reinterpret_cast<cd *>(rtmp);  // [nsel][DEG + 2]: coefficients, then w
        uint32_t *rflag = reinterpret_cast<uint32_t *>(pco + (size_t)nsel * (DEG + 2));  // [nsel][DEG]
        int *pok = reinterpret_cast<int *>(rflag + (size_t)nsel * DEG);                  // [nsel]
        int *psl = pok + nsel;                                                           // [nsel]
        // binary lenses: one lane per (new point, coefficient), dense over the
        // first two warps; each lane forms its point's source position and one
        // coefficient (lens_poly2_coef), a chain half as long as the whole
        // polynomial on one lane
        if constexpr (NL == 2) {
          for (int idx = tid; idx < nsel * (DEG + 1); idx += ES_THREADS) {
            const int j = idx / (DEG + 1), m = idx - j * (DEG + 1);
            const int k = NEWK[j], slot = Lcur + j;
            const int sl = S.ORD[k], sr = S.ORD[k + 1];
            const double th = 0.5 * (S.TH[sl] + S.TH[sr]);
            double sn, cs;
            sincos(th, &sn, &cs);
            const cd w = mk(__dadd_rn(__dmul_rn(I.rho, cs), I.w0.x), __dadd_rn(__dmul_rn(I.rho, sn), I.w0.y));
            pco[(size_t)j * (DEG + 2) + m] = lens_poly2_coef(I.L, w, m);
            if (m < DEG)  // warm start from the left neighbour's rows with the fixed jitter
              S.Z[(size_t)slot * DEG + m] =
                  S.Z[(size_t)sl * DEG + m] + mk(1e-6 * ((m & 1) ? 0.5 : -0.5), 1e-6 * ((m & 2) ? 0.5 : -0.5));
            if (m == 0) {
              S.TH[slot] = th;
              psl[j] = sl;
              pco[(size_t)j * (DEG + 2) + DEG + 1] = w;
            }
          }
        } else {
          // one thread per new point, dense over the first warps: FP64 work
          // spread over every warp costs each warp the whole instruction stream
          for (int j = tid; j < nsel; j += ES_THREADS) {
            const int k = NEWK[j], slot = Lcur + j;
            const int sl = S.ORD[k], sr = S.ORD[k + 1];
            const double th = 0.5 * (S.TH[sl] + S.TH[sr]);
            S.TH[slot] = th;
            psl[j] = sl;
            double sn, cs;
            sincos(th, &sn, &cs);
            const cd w = mk(__dadd_rn(__dmul_rn(I.rho, cs), I.w0.x), __dadd_rn(__dmul_rn(I.rho, sn), I.w0.y));
            cd p[DEG + 1];
            lens_poly<NL>(I.L, w, p);
#pragma unroll
            for (int i = 0; i <= DEG; ++i) pco[(size_t)j * (DEG + 2) + i] = p[i];
            pco[(size_t)j * (DEG + 2) + DEG + 1] = w;
            // warm start from the left neighbour's rows with the fixed jitter
            // (extended_source.py:79-98, 128-129)
#pragma unroll
            for (int i = 0; i < DEG; ++i)
              S.Z[(size_t)slot * DEG + i] =
                  S.Z[(size_t)sl * DEG + i] + mk(1e-6 * ((i & 1) ? 0.5 : -0.5), 1e-6 * ((i & 2) ? 0.5 : -0.5));
          }
        }
        __syncthreads();
        // The FP32 stage on a lane group per new point, one lane per root,
        // every root updated from the previous iterate (simultaneous Aberth
        // steps); the FP32 stopping rule of the reference's iteration.  Up to
        // 5 FP64 Newton steps per root follow, so the compensated stage is not
        // needed; a group that does not converge goes to the FP64 fallback.
        {
          constexpr int FG = RefGroup<DEG>::G;
          const int lg = tid & (FG - 1);
          const unsigned gmask = (FG == 32) ? 0xffffffffu : (((1u << FG) - 1u) << ((tid & 31) - lg));
          for (int j = tid / FG; j < nsel; j += ES_THREADS / FG) {
            const int slot = Lcur + j;
            cf ph[DEG + 1];
            float alpha[DEG + 1];
#pragma unroll
            for (int q = 0; q <= DEG; ++q) {
              ph[q] = tof(pco[(size_t)j * (DEG + 2) + q]);
              alpha[q] = cabs(ph[q]) * fmaf(3.8284271247461900976f, (float)q, 1.0f);
            }
            cf zr = lg < DEG ? tof(S.Z[(size_t)slot * DEG + lg]) : mkf(0.0f, 0.0f);
            bool done = lg >= DEG;
            int it = 0;
            for (; it < 64; ++it) {
              cf zall[DEG];
#pragma unroll
              for (int q = 0; q < DEG; ++q)
                zall[q] = mkf(__shfl_sync(gmask, zr.x, q, FG), __shfl_sync(gmask, zr.y, q, FG));
              if (!done) {
                const float az = cabs(zr);
                const bool rev = az > 1.0f;
                const cf x = rev ? crecip(zr) : zr;
                cf h, hd;
                float b;
                horner_pair<DEG>(ph, alpha, x, rev ? 1.0f / az : az, rev, h, hd, b);
                if (cabs(h) > CGB_EPS32 * b) {
                  cf sum = mkf(0.0f, 0.0f);
#pragma unroll
                  for (int q = 0; q < DEG; ++q)
                    if (q != lg) sum = sum + crecip(zr - zall[q]);
                  cf corr;
                  if (rev) {
                    const cf z2h = (zr * zr) * h;
                    const cf d = zr * h;
                    corr = cdiv(z2h, mkf(d.x * DEG, d.y * DEG) - hd - z2h * sum);
                  } else {
                    corr = cdiv(h, hd - h * sum);
                  }
                  zr = zr - corr;
                } else {
                  done = true;
                }
              }
              if (__all_sync(gmask, done)) break;
            }
            const bool ok = __all_sync(gmask, done && isfinite(zr.x) && isfinite(zr.y));
            // S^2 of this root for the polish's error model (newton_polish_root),
            // handed over in the point's flag slots
            float sep = 0.0f;
#pragma unroll
            for (int q = 0; q < DEG; ++q) {
              const cf zq = mkf(__shfl_sync(gmask, zr.x, q, FG), __shfl_sync(gmask, zr.y, q, FG));
              if (q != lg) sep += rsqrtf(norm2(zr - zq));
            }
            if (lg < DEG) {
              S.Z[(size_t)slot * DEG + lg] = tod(zr);
              rflag[(size_t)j * DEG + lg] = __float_as_uint(sep * sep);
            }
            if (lg == 0) {
              pok[j] = ok ? 1 : 0;
              if (P.dbg) {
                atomicAdd(&dbg_ref[5], it + 1);
                atomicAdd(&dbg_ref[6], 1);
              }
            }
          }
        }
        if (P.dbg && lane == 0) dbg_arr[warp] = clock64();
        __syncthreads();
        if (P.dbg && tid == 0) {
          const long long t = last_arrival();
          dbg_b[1] += t - tb;
          tb = t;
        }
        if (P.dbg) __syncthreads();
        for (int idx = tid; idx < nsel * DEG; idx += ES_THREADS) {
          const int j = idx / DEG, i = idx - j * DEG, slot = Lcur + j;
          uint32_t f = 0;
          if (pok[j]) {
            cd p[DEG + 1];
#pragma unroll
            for (int q = 0; q <= DEG; ++q) p[q] = pco[(size_t)j * (DEG + 2) + q];
            cd z = S.Z[(size_t)slot * DEG + i];
            if (newton_polish_root<DEG, 5>(p, z, GRAD ? INFINITY : __uint_as_float(rflag[idx]))) f |= 1u;
            S.Z[(size_t)slot * DEG + i] = z;
            double r, d;
            lens_filter<NL>(I.L, z, pco[(size_t)j * (DEG + 2) + DEG + 1], r, d);
            if (r < 1e-6) f |= 2u;
            if (d > 0) f |= 4u;
            if (d == 0) f |= 8u;
            if (r > 1e-6 / 30 && r < 1e-6 * 30) f |= 16u;
          }
          rflag[idx] = f;
        }
        if (P.dbg && lane == 0) dbg_arr[warp] = clock64();
        __syncthreads();
        if (P.dbg && tid == 0) {
          const long long t = last_arrival();
          dbg_b[2] += t - tb;
          tb = t;
        }
        if (P.dbg) __syncthreads();
        // per-point checks and labelling on the same lane groups (lane r: root r
        // of the new point, row r of its left neighbour)
        {
          constexpr int FG = RefGroup<DEG>::G;
          const int lg = tid & (FG - 1);
          const unsigned gmask = (FG == 32) ? 0xffffffffu : (((1u << FG) - 1u) << ((tid & 31) - lg));
          const int gbase = (tid & 31) - lg;
          const uint32_t all = (1u << DEG) - 1u;
          for (int j = tid / FG; j < nsel; j += ES_THREADS / FG) {
            const int slot = Lcur + j, sl = psl[j];
            cd *zrow = S.Z + (size_t)slot * DEG;
            uint32_t f = lg < DEG ? rflag[j * DEG + lg] : 1u;
            auto distinct = [&]() {  // no two roots closer than 1e-7 of the largest modulus
              // the largest |z|^2 by a shuffle tree (lane r: root r), then the
              // DEG (DEG - 1) / 2 pairs dealt evenly over the group's lanes:
              // the same exact comparisons on a shorter FP64 chain per lane
              double scale = lg < DEG ? norm2(zrow[lg]) : 0.0;
#pragma unroll
              for (int o = 1; o < FG; o <<= 1) scale = fmax(scale, __shfl_xor_sync(gmask, scale, o, FG));
              bool sep = true;
              for (int pr = lg; pr < DEG * (DEG - 1) / 2; pr += FG) {
                int a = 0, rem = pr;
                while (rem >= DEG - 1 - a) rem -= DEG - 1 - (a++);
                if (norm2(zrow[a] - zrow[a + 1 + rem]) < 1e-14 * scale) sep = false;
              }
              return __all_sync(gmask, sep);
            };
            bool ok = pok[j] != 0 && __all_sync(gmask, (f & 1u) != 0);
            if (ok) ok = distinct();  // (Newton alone may merge a near-double pair)
            bool group_fb = false;
            if (!ok) {
              // FP64 fallback on the group first: simultaneous Aberth steps from
              // the left neighbour's roots plus the jitter (the FP64 path's own
              // start), one lane per root; then the filter per lane as above
              cd p[DEG + 1];
#pragma unroll
              for (int q = 0; q <= DEG; ++q) p[q] = pco[(size_t)j * (DEG + 2) + q];
              cd zr = lg < DEG ? S.Z[(size_t)sl * DEG + lg] +
                                     mk(1e-6 * ((lg & 1) ? 0.5 : -0.5), 1e-6 * ((lg & 2) ? 0.5 : -0.5))
                               : mk(0.0, 0.0);
              if (aberth64_group<DEG, FG>(p, zr, min(P.itmax, 64), gmask)) {
                if (lg < DEG) zrow[lg] = zr;
                __syncwarp(gmask);
                if (distinct()) {
                  f = 1u;
                  if (lg < DEG) {
                    double r, d;
                    lens_filter<NL>(I.L, zr, pco[(size_t)j * (DEG + 2) + DEG + 1], r, d);
                    if (r < 1e-6) f |= 2u;
                    if (d > 0) f |= 4u;
                    if (d == 0) f |= 8u;
                    if (r > 1e-6 / 30 && r < 1e-6 * 30) f |= 16u;
                  }
                  ok = group_fb = true;
                }
              }
            }
            if (ok) {
              if (group_fb && lg == 0) flags |= CGB_ST_FALLBACK;
              const uint32_t mkb = (__ballot_sync(gmask, lg < DEG && (f & 2u)) >> gbase) & all;
              const uint32_t pp = (__ballot_sync(gmask, lg < DEG && (f & 4u)) >> gbase) & all;
              const uint32_t zp = (__ballot_sync(gmask, lg < DEG && (f & 8u)) >> gbase) & all;
              if (lg < DEG && (f & 16u)) flags |= CGB_ST_AMBIGUOUS;
              if (lg == 0) {
                S.MK[slot] = (uint16_t)mkb;
                S.PP[slot] = (uint16_t)pp;
                S.ZP[slot] = (uint16_t)zp;
              }
            } else if (lg == 0) {  // the mixed solver's FP64 fallback, then the filter here
              flags |= CGB_ST_FALLBACK;
              cd p[DEG + 1], z[DEG], warm[DEG];
#pragma unroll
              for (int q = 0; q <= DEG; ++q) p[q] = pco[(size_t)j * (DEG + 2) + q];
              // the FP64 path's own start: the left neighbour's roots plus the jitter
#pragma unroll
              for (int i = 0; i < DEG; ++i)
                warm[i] = S.Z[(size_t)sl * DEG + i] + mk(1e-6 * ((i & 1) ? 0.5 : -0.5), 1e-6 * ((i & 2) ? 0.5 : -0.5));
              if (aberth64_fallback<DEG>(p, z, P.itmax, warm) < 0) flags |= CGB_ST_NOCONV;
              const cd w = pco[(size_t)j * (DEG + 2) + DEG + 1];
              uint16_t mkb = 0, pp = 0, zp = 0;
#pragma unroll
              for (int i = 0; i < DEG; ++i) {
                zrow[i] = z[i];
                double r, d;
                lens_filter<NL>(I.L, z[i], w, r, d);
                if (r < 1e-6) mkb |= 1u << i;
                if (r > 1e-6 / 30 && r < 1e-6 * 30) flags |= CGB_ST_AMBIGUOUS;
                if (d > 0) pp |= 1u << i;
                if (d == 0) zp |= 1u << i;
              }
              S.MK[slot] = mkb;
              S.PP[slot] = pp;
              S.ZP[slot] = zp;
            }
            __syncwarp(gmask);
            // step_map on the group: lane r finds row r's nearest and second
            // nearest new root; clear when every row's nearest is nearer than
            // half its second nearest and no two rows share one
            // (squared distances are >= +0, so their bit patterns order as
            // unsigned integers, any NaN above +inf: the comparisons run on
            // the integer pipe)
            int best = 0;
            bool clear = true;
            if (lg < DEG) {
              const cd ar = S.Z[(size_t)sl * DEG + lg];
              unsigned long long d1 = (unsigned long long)__double_as_longlong(INFINITY), d2 = d1;
#pragma unroll
              for (int q = 0; q < DEG; ++q) {
                const unsigned long long d = (unsigned long long)__double_as_longlong(norm2(zrow[q] - ar));
                if (d < d1) {
                  d2 = d1;
                  d1 = d;
                  best = q;
                } else if (d < d2) {
                  d2 = d;
                }
              }
              clear = __longlong_as_double((long long)d1) < 0.25 * __longlong_as_double((long long)d2);
            }
            uint32_t bits = lg < DEG ? (1u << best) : 0u;
#pragma unroll
            for (int o = FG >> 1; o > 0; o >>= 1) bits |= __shfl_xor_sync(gmask, bits, o, FG);
            const bool amb = !__all_sync(gmask, clear) || bits != all;
            uint64_t m = 0;
#pragma unroll
            for (int q = 0; q < DEG; ++q) m = perm_set(m, q, __shfl_sync(gmask, best, q, FG));
            if (lg == 0) {
              if (amb && !P.nearest) {  // labelled below by the reference's warm start, on a lane group
                S.USED[atomicAdd(&nlist_sh, 1)] = (uint64_t)slot | ((uint64_t)sl << 16);
              } else {
                if (amb) m = greedy_match<DEG>(S.Z + (size_t)sl * DEG, zrow);
                apply_rows<DEG>(zrow, S.MK[slot], S.PP[slot], S.ZP[slot], m);
              }
            }
          }
        }
      } else
      for (int j = tid; j < nsel; j += ES_THREADS) {  // one thread per new point, dense
        const int k = NEWK[j];
        const int slot = Lcur + j;
        const int sl = S.ORD[k], sr = S.ORD[k + 1];
        const double th = 0.5 * (S.TH[sl] + S.TH[sr]);
        S.TH[slot] = th;
        // warm start from the left neighbour's rows (extended_source.py:79-98,
        // 128-129); the row order is the reference's warm-start labelling
        solve_limb_point<NL, PREC, !GRAD>(P, I, th, S.Z + (size_t)slot * DEG, S.Z + (size_t)sl * DEG, S.MK[slot],
                                   S.PP[slot], S.ZP[slot], flags);
        bool amb;
        const uint64_t m = step_map<DEG>(S.Z + (size_t)sl * DEG, S.Z + (size_t)slot * DEG, amb);
        if (amb && !P.nearest)  // labelled below by the reference's warm start, on a lane group
          S.USED[atomicAdd(&nlist_sh, 1)] = (uint64_t)slot | ((uint64_t)sl << 16);
        else
          apply_rows<DEG>(S.Z + (size_t)slot * DEG, S.MK[slot], S.PP[slot], S.ZP[slot], m);
      }
      if (P.dbg && lane == 0) dbg_arr[warp] = clock64();
      __syncthreads();
      if (P.dbg && tid == 0) {
        const long long t = last_arrival();
        dbg_b[PREC == MIXED ? 3 : 1] += t - tb;
        tb = t;
      }
      if (P.dbg) __syncthreads();  // keep the arrival clocks until read
      {
        uint64_t ident = 0;
        for (int t = 0; t < DEG; ++t) ident = perm_set(ident, t, t);
        for (int e = tid / RG; e < nlist_sh; e += ES_THREADS / RG) {
          const int slot = (int)(S.USED[e] & 0xffffu), sl = (int)((S.USED[e] >> 16) & 0xffffu);
          int its;
          const uint64_t m = warm_map_ref_group<NL>(P, I, S.TH[slot], S.Z + (size_t)sl * DEG, ident,
                                                    S.Z + (size_t)slot * DEG, true, its);
          if ((tid & (RG - 1)) == 0) {
            apply_rows<DEG>(S.Z + (size_t)slot * DEG, S.MK[slot], S.PP[slot], S.ZP[slot], m);
            if (P.dbg) {
              atomicAdd(&dbg_ref[3], 1);
              atomicAdd(&dbg_ref[4], its);
            }
          }
        }
      }
      if (P.dbg && lane == 0) dbg_arr[warp] = clock64();
      __syncthreads();
      if (P.dbg && tid == 0) {
        const long long t = last_arrival();
        dbg_b[4] += t - tb;
        tb = t;
      }
      if (P.dbg) __syncthreads();  // keep the arrival clocks until read
      // the intervals on either side of each new point (one thread per point),
      // at their limb positions after the insertion; the rest of the ranked
      // list keeps its order, its positions shift past the new points
      const int nb = 2 * nsel;
      int nbs = 1;
      while (nbs < nb) nbs <<= 1;
      long long *NBV = reinterpret_cast<long long *>(rtmp);  // [nbs] new intervals
      uint16_t *NBP = reinterpret_cast<uint16_t *>(NBV + nbs);
      long long *MGV = reinterpret_cast<long long *>(rtmp + (((size_t)nbs * 10 + 15) & ~(size_t)15));  // merged
      uint16_t *MGP = reinterpret_cast<uint16_t *>(MGV + (ngap + nsel));
      // one lane per new interval (e = 2 j: left of new point j, 2 j + 1: right)
      for (int e = tid; e < nbs; e += ES_THREADS) {
        if (e < nb) {
          const int j = e >> 1, side = e & 1, k = NEWK[j], m = Lcur + j;
          const double len = side ? interval_len<DEG>(S, m, S.ORD[k + 1]) : interval_len<DEG>(S, S.ORD[k], m);
          NBV[e] = __double_as_longlong(len);
          NBP[e] = (uint16_t)(k + j + side);
        } else {
          NBV[e] = -1ll;
          NBP[e] = 0;
        }
      }
      for (int r = nsel + tid; r < ngap; r += ES_THREADS) SLP[r] = (uint16_t)(SLP[r] + S.SCAN[SLP[r]]);
      // insertion: old position k -> k + (#selected before k); new point after k
      for (int k = tid; k < Lcur; k += ES_THREADS) {
        const int before = S.SCAN[k];
        S.ORD2[k + before] = S.ORD[k];
        if (k < ngap && S.KEY[k] != 0.0) S.ORD2[k + before + 1] = (uint16_t)(Lcur + before);
      }
      __syncthreads();
      for (int k = tid; k < Lcur + nsel; k += ES_THREADS) S.ORD[k] = S.ORD2[k];
      bitonic_sort_desc(NBV, NBP, nbs);  // starts after the barrier above, ends with one
      {
        // merge the rest of the ranked list (ma entries) with the new intervals
        // (nb): each entry's place = its own index + the entries of the other
        // list ranked before it (keys are distinct: positions are)
        const long long *AV = SLV + nsel;
        const uint16_t *AP = SLP + nsel;
        const int ma = ngap - nsel;
        for (int i = tid; i < ma + nb; i += ES_THREADS) {
          const bool fromA = i < ma;
          const long long v = fromA ? AV[i] : NBV[i - ma];
          const int pos = fromA ? AP[i] : NBP[i - ma];
          const long long *OV = fromA ? NBV : AV;
          const uint16_t *OP = fromA ? NBP : AP;
          int lo = 0, hi = fromA ? nb : ma;
          while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (OV[mid] > v || (OV[mid] == v && OP[mid] > pos)) lo = mid + 1; else hi = mid;
          }
          const int at = (fromA ? i : i - ma) + lo;
          MGV[at] = v;
          MGP[at] = (uint16_t)pos;
        }
        __syncthreads();
        for (int i = tid; i < ma + nb; i += ES_THREADS) {
          SLV[i] = MGV[i];
          SLP[i] = MGP[i];
        }
      }
      Lcur += nsel;
      if (P.dbg && lane == 0) dbg_arr[warp] = clock64();
      __syncthreads();
      if (P.dbg && tid == 0) {
        const long long t = last_arrival();
        dbg_b[5] += t - tb;
        tb = t;
      }
      if (P.dbg) __syncthreads();
    }
    const int L = Lcur;
    if (P.dbg && tid == 0) clk[2] = clock64();

    // ---- C: final chained matching (extended_source.py:150-151) ----
    chain_match<DEG>(S, L);
    if (P.dbg && tid == 0) clk[3] = clock64();

    // ---- D: segments (extended_source.py:251-309) ----
    TrackView<DEG> V{&S};
    if (tid == 0) {
      MergeState &M = *S.M;
      M.nseg = 0;
      M.nclosed = 0;
      M.flags = 0;
      M.all_closed = 1;
      for (int c = 0; c < N_CONTOURS; ++c) {
        M.npieces[c] = 0;
        M.cnpts[c] = 0;
        M.cpar[c] = 0;
      }
    }
    __syncthreads();
    // per track: closed?  (warp t handles track t)
    for (int t = warp; t < DEG; t += ES_WARPS) {
      bool allreal = true;
      for (int k = lane; k < L; k += 32) {
        int slot = S.ORD[k], row = perm_get(S.PERM[k], t);
        allreal &= ((S.MK[slot] >> row) & 1u) != 0;
      }
      allreal = __all_sync(0xffffffffu, allreal);
      if (lane == 0) {
        bool closed = allreal && cabs(V.at(t, 0) - V.at(t, L - 1)) < 1e-5;
        if (closed) {
          int q = atomicAdd(&S.M->nclosed, 1);
          S.M->closed_tracks[q] = t;
        } else {
          atomicAnd(&S.M->all_closed, 0);
        }
      }
    }
    __syncthreads();
    // Change points of the open tracks (extended_source.py:156-216), found in
    // parallel as bits per (track, position k = 0..L): START (a part starts at
    // k), END (a part ends at k), NZ (a real, non-zero image at k).  The bits live
    // in the candidate lists' storage, free after the chained matching.
    const int W = (L + 1 + 63) >> 6;
    uint64_t *bits = S.CAND;
    const bool open_tracks = !S.M->all_closed;
    if (open_tracks) {
      for (int i = tid; i < 3 * DEG * W; i += ES_THREADS) bits[i] = 0ull;
      __syncthreads();
      for (int idx = tid; idx < DEG * (L + 1); idx += ES_THREADS) {
        const int t = idx / (L + 1), k = idx - t * (L + 1);
        auto real_at = [&](int kk) {
          int slot = S.ORD[kk], row = perm_get(S.PERM[kk], t);
          return (int)((S.MK[slot] >> row) & 1u);
        };
        auto par_at = [&](int kk) {
          int slot = S.ORD[kk], row = perm_get(S.PERM[kk], t);
          if (!((S.MK[slot] >> row) & 1u)) return 0;
          if ((S.ZP[slot] >> row) & 1u) return 0;
          return ((S.PP[slot] >> row) & 1u) ? 1 : -1;
        };
        int ch, dm;
        if (k == 0) {
          ch = real_at(0);
          dm = real_at(0);
        } else if (k == L) {
          ch = real_at(L - 1);
          dm = real_at(L - 1) ? -1 : 0;
        } else {
          int r0 = real_at(k - 1), r1 = real_at(k);
          cd z0 = r0 ? V.at(t, k - 1) : mk(0, 0), z1 = r1 ? V.at(t, k) : mk(0, 0);
          cd dz = z1 - z0;
          bool jump = dz.x * dz.x + dz.y * dz.y > 0.1 * 0.1;
          dm = r1 - r0;
          ch = jump || (par_at(k) - par_at(k - 1) != 0) || (dm != 0);
        }
        const unsigned long long b = 1ull << (k & 63);
        if (ch && dm >= 0) atomicOr((unsigned long long *)&bits[(0 * DEG + t) * W + (k >> 6)], b);
        if (ch && dm <= 0) atomicOr((unsigned long long *)&bits[(1 * DEG + t) * W + (k >> 6)], b);
        if (k < L && real_at(k)) {
          const cd zz = V.at(t, k);
          if (zz.x != 0.0 || zz.y != 0.0) atomicOr((unsigned long long *)&bits[(2 * DEG + t) * W + (k >> 6)], b);
        }
      }
    }
    __syncthreads();
    if (tid == 0) {
      MergeState &M = *S.M;
      // closed tracks in track order
      for (int i = 1; i < M.nclosed; ++i)
        for (int j = i; j > 0 && M.closed_tracks[j - 1] > M.closed_tracks[j]; --j) {
          int x = M.closed_tracks[j];
          M.closed_tracks[j] = M.closed_tracks[j - 1];
          M.closed_tracks[j - 1] = x;
        }
      if (open_tracks) {
        // split open tracks; parts ordered as argsort(nonempty)[::-1]:
        // non-empty parts by descending (track, part)
        int nseg_keep = 3 * DEG;
        int cand = 0;
        for (int t = DEG - 1; t >= 0; --t) {
          bool closed = false;
          for (int i = 0; i < M.nclosed; ++i) closed |= M.closed_tracks[i] == t;
          int starts[10], ends[10], ns = 0, ne = 0;
          if (!closed) {
            for (int w = 0; w < W && ns < 10; ++w)
              for (uint64_t x = bits[(0 * DEG + t) * W + w]; x && ns < 10; x &= x - 1)
                starts[ns++] = (w << 6) + __ffsll((long long)x) - 1;
            for (int w = 0; w < W && ne < 10; ++w)
              for (uint64_t x = bits[(1 * DEG + t) * W + w]; x && ne < 10; x &= x - 1)
                ends[ne++] = (w << 6) + __ffsll((long long)x) - 1;
          }
          for (int q = 9; q >= 0; --q) {
            int l = q < ns ? starts[q] : 0, r = q < ne ? ends[q] : 0;
            if (l == 0 && r == 0) continue;
            int cnt = 0;  // real, non-zero images in [l, r)
            for (int w = l >> 6; l < r && w <= ((r - 1) >> 6); ++w) {
              uint64_t x = bits[(2 * DEG + t) * W + w];
              if (w == (l >> 6)) x &= ~0ull << (l & 63);
              if (w == ((r - 1) >> 6) && ((r - 1) & 63) != 63) x &= (2ull << ((r - 1) & 63)) - 1ull;
              cnt += __popcll(x);
            }
            if (cnt < 2) continue;
            if (cand < nseg_keep) {
              Segment &sg = M.seg[cand];
              sg.t = (int16_t)t;
              sg.l = (int16_t)l;
              sg.r = (int16_t)r;
              int slot = S.ORD[l], row = perm_get(S.PERM[l], t);
              sg.par = ((S.ZP[slot] >> row) & 1u) ? 0 : (((S.PP[slot] >> row) & 1u) ? 1 : -1);
              sg.alive = 1;
              sg.len = 0.0;
            }
            ++cand;
          }
        }
        if (cand > nseg_keep) M.flags |= CGB_ST_MERGE;
        int nfill = min(cand, nseg_keep);
        for (int i = nfill; i < nseg_keep; ++i) {
          M.seg[i] = Segment{0, 0, 0, 0, 0.0, 0};
        }
        M.nseg = nseg_keep;
      }
    }
    __syncthreads();
    if (open_tracks) {
      // path length of every segment: one warp each
      for (int q = warp; q < S.M->nseg; q += ES_WARPS) {
        const Segment sg = S.M->seg[q];
        if (!sg.alive) continue;
        double len = 0.0;
        for (int k = sg.l + lane; k + 1 < sg.r; k += 32) len += cabs(V.at(sg.t, k + 1) - V.at(sg.t, k));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) len += __shfl_xor_sync(0xffffffffu, len, o);
        if (lane == 0) S.M->seg[q].len = len;
      }
      __syncthreads();
      if (tid == 0) merge_segments<DEG>(S, L);
    }
    __syncthreads();
    if (P.dbg && tid == 0) clk[4] = clock64();

    // ---- E: contour point lists ----
    if (tid == 0) {
      MergeState &M = *S.M;
      int n = 0, c = 0;
      for (int i = 0; i < M.nclosed; ++i) {
        int t = M.closed_tracks[i];
        cstart[c] = n;
        int slot = S.ORD[0], row = perm_get(S.PERM[0], t);
        cpar[c] = ((S.ZP[slot] >> row) & 1u) ? 0 : (((S.PP[slot] >> row) & 1u) ? 1 : -1);
        n += L + 1;
        ++c;
      }
      for (int k = 0; k < N_CONTOURS; ++k) {
        if (M.cnpts[k] == 0) continue;
        cstart[c] = n;
        cpar[c] = M.cpar[k];
        int np = M.cnpts[k];
        int cap = 4 * L;
        n += (np + 1 <= cap) ? np + 1 : np;  // closing point unless the buffer is full
        ++c;
      }
      cstart[c] = n;
      nsel_sh = c;
      if (n > P.CPcap) M.flags |= CGB_ST_CAPACITY;
    }
    __syncthreads();
    const int ncont = nsel_sh;
    // fill CP in parallel: closed tracks
    {
      MergeState &M = *S.M;
      for (int i = 0; i < M.nclosed; ++i) {
        int t = M.closed_tracks[i];
        int base = cstart[i];
        for (int k = tid; k <= L; k += ES_THREADS) {
          int kk = k < L ? k : 0;
          if (base + k < P.CPcap) S.CP[base + k] = V.cp(t, kk);
        }
      }
      if (tid == 0) {
        int c = M.nclosed;
        for (int k = 0; k < N_CONTOURS; ++k) {
          if (M.cnpts[k] == 0) continue;
          int base = cstart[c], n = cstart[c + 1] - base, i = 0;
          for (int q = 0; q < M.npieces[k] && i < n; ++q) {
            const Piece &pc = M.pieces[k][q];
            for (int u = 0; u < pc.r - pc.l && i < n; ++u, ++i) {
              int kk = pc.dir > 0 ? pc.l + u : pc.r - 1 - u;
              if (base + i < P.CPcap) S.CP[base + i] = V.cp(pc.t, kk);
            }
          }
          if (i < n && base + i < P.CPcap) S.CP[base + i] = S.CP[base];  // closing point
          ++c;
        }
      }
    }
    __syncthreads();
    const int ntot = min(cstart[ncont], P.CPcap);
    if (P.dbg && tid == 0) clk[5] = clock64();

    // ---- F: integrals ----
    for (int c = tid; c < MAX_CLOSED + N_CONTOURS; c += ES_THREADS) {
      for (int w = 0; w < ES_WARPS; ++w) {
        contour_acc[w][c] = 0.0;
        if (GRAD) cgr_w[w][c][0] = cgr_w[w][c][1] = 0.0;
      }
      cgr[c][0] = cgr[c][1] = 0.0;
    }
    if (GRAD)
      for (int k = tid; k < NK_MAX * ES_MAX_WARPS; k += ES_THREADS) pgr_w[k / NK_MAX][k % NK_MAX] = 0.0;
    if (P.ld) {
      // centroids (sum over all points incl. the closing point) / count
      for (int c = warp; c < ncont; c += ES_WARPS) {
        cd s = mk(0, 0);
        int b = cstart[c], e = min(cstart[c + 1], ntot);
        for (int i = b + lane; i < e; i += 32) s = s + S.Z[S.CP[i]];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
          s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
        }
        if (lane == 0) centroid[c] = mk(s.x / (e - b), s.y / (e - b));
      }
    }
    __syncthreads();
    if (P.ld) {
      // groups of G lanes per contour point (G = P.ld_group), each lane taking
      // every G-th node: I_c = sum_i P_i wx_i + Q_i wy_i (trapezoid weights)
      const int G = P.ld_group, groups = ES_THREADS / G, r = tid % G, gid = tid / G;
      const LdConst ldk = ld_const<NL>(I);
      const int iters = (ntot + groups - 1) / groups;
      int c = 0;
      for (int it = 0; it < iters; ++it) {
        const int i = it * groups + gid;
        const bool valid = i < ntot;
        cd pq = mk(0, 0);
        double wx = 0.0, wy = 0.0;
        if (valid) {
          while (i >= cstart[c + 1]) ++c;
          const int b = cstart[c], e = min(cstart[c + 1], ntot);
          cd zc = S.Z[S.CP[i]];
          cd zp = i > b ? S.Z[S.CP[i - 1]] : zc, zn = i + 1 < e ? S.Z[S.CP[i + 1]] : zc;
          wx = 0.5 * (zn.x - zp.x);
          wy = 0.5 * (zn.y - zp.y);
          pq = (PREC == MIXED) ? ld_point_mixed<NL>(P, I, ldk, zc, S.TH[S.CP[i] / DEG], centroid[c], r, G, glf)
                               : ld_point_fp64<NL>(P, I, zc, centroid[c], r, G);
        }
        for (int o = G >> 1; o > 0; o >>= 1) {
          pq.x += __shfl_xor_sync(0xffffffffu, pq.x, o);
          pq.y += __shfl_xor_sync(0xffffffffu, pq.y, o);
        }
        warp_run_add(valid ? c : -1, (valid && r == 0) ? pq.x * wx + pq.y * wy : 0.0, contour_acc[warp]);
      }
    } else {
      // uniform: 1/2 sum (x_i + x_{i+1})/2 (y_{i+1} - y_i) - (y_i + y_{i+1})/2 (x_{i+1} - x_i)
      int c = 0;
      for (int base = warp * 32; base < ntot; base += ES_THREADS) {  // warp-uniform trip count
        const int i = base + lane;
        double v = 0.0;
        int key = -1;
        if (i < ntot) {
          while (i >= cstart[c + 1]) ++c;
          key = c;
          const int e = min(cstart[c + 1], ntot);
          if (i + 1 < e) {
            const cd a = S.Z[S.CP[i]], bq = S.Z[S.CP[i + 1]];
            v = 0.25 * ((a.x + bq.x) * (bq.y - a.y) - (a.y + bq.y) * (bq.x - a.x));
          }
        }
        warp_run_add(key, v, contour_acc[warp]);
      }
    }
    __syncthreads();
    if (GRAD)
      es_backward<NL, PREC>(P, S, I, ncont, ntot, cstart, cpar, centroid, contour_acc, cgr, cgr_w, pgr_w, &tot_sh, pi,
                            mag, glf);
    if (tid == 0 && !GRAD) {
      double tot = 0.0;
      double *dbg = P.dbg ? P.dbg + (size_t)pi * ES_DBG_STRIDE(P.Lcap) : nullptr;
      for (int c = 0; c < ncont; ++c) {
        double s = 0.0;
        for (int w = 0; w < ES_WARPS; ++w) s += contour_acc[w][c];
        tot += s * cpar[c];
        if (dbg && c < 13) {
          dbg[3 + 4 * c] = cstart[c];
          dbg[4 + 4 * c] = cstart[c + 1] - cstart[c];
          dbg[5 + 4 * c] = cpar[c];
          dbg[6 + 4 * c] = s;
        }
      }
      if (dbg) {
        dbg[0] = L;
        dbg[1] = ncont;
        dbg[2] = S.M->flags;
        clk[6] = clock64();
        for (int c = 1; c < 7; ++c) dbg[ES_DBG_CLK + c - 1] = (double)(clk[c] - clk[c - 1]);
        // faithful solves: A (chain repair) count + 1000 * first-point iterations; B count + 1000 * iterations
        dbg[ES_DBG_CLK + 6] = dbg_ref[1] + 1000.0 * (dbg_ref[0] + dbg_ref[2]);
        dbg[ES_DBG_CLK + 7] = dbg_ref[3] + 1000.0 * dbg_ref[4];
      }
      mag[pi] = fabs(tot) / (3.14159265358979323846 * I.rho * I.rho);
    }
    if (tid == 0) atomicOr(&sflags, S.M->flags);
    atomicOr(&sflags, flags);
    __syncthreads();
    if (tid == 0 && status) status[pi] = route ? (status[pi] | sflags) : sflags;
    if (P.dbg) {
      for (int k = tid; k < L; k += ES_THREADS) P.dbg[(size_t)pi * ES_DBG_STRIDE(P.Lcap) + ES_DBG_HEAD + k] = S.TH[S.ORD[k]];
      if (tid < ES_DBG_SUB) P.dbg[(size_t)pi * ES_DBG_STRIDE(P.Lcap) + ES_DBG_HEAD + P.Lcap + tid] = (double)dbg_b[tid];
      if (tid < 2) P.dbg[(size_t)pi * ES_DBG_STRIDE(P.Lcap) + ES_DBG_HEAD + P.Lcap + ES_DBG_SUB + tid] = dbg_ref[5 + tid];
    }
    __syncthreads();
  }
}

template <int NL, int PREC, bool GRAD>
cudaError_t launch_es_variant(const EsParams &P, const cd *w0, const int64_t *index, const uint8_t *route, int64_t n,
                              double *mag, uint32_t *status, int grid, cudaStream_t stream) {
  size_t smem = es_smem_bytes(P, NL, GRAD);
  auto k = es_kernel<NL, PREC, GRAD>;
  // 0 = automatic: at npts_limb <= ~256 a forward evaluation's phases keep few
  // threads busy, and 128-thread CTAs (four per SM by registers) measured 5 %
  // faster than 256 on the 4096-curve workload; the adjoint measured faster
  // at 256 (15 %)
  const int threads = P.threads > 0 ? P.threads : ((!GRAD && P.Lcap <= 256) ? 128 : ES_MAX_THREADS);
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (grid <= 0) {  // persistent: as many CTAs as fit on the device
    int dev = 0, sms = 1, per_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, threads, smem);
    grid = sms * (per_sm > 0 ? per_sm : 1);
  }
  if (P.perm0 && !P.nearest) {
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    es_first_order_kernel<NL, PREC, !GRAD><<<sms * 8, FO_THREADS, 0, stream>>>(P, w0, index, route, n,
                                                                         const_cast<uint64_t *>(P.perm0));
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    // programmatic dependent launch: the contour kernel starts while the
    // ordering kernel runs and waits for it only where it reads perm0
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, P, w0, index, route, n, mag, status);
  }
  k<<<grid, threads, smem, stream>>>(P, w0, index, route, n, mag, status);
  return cudaGetLastError();
}

}  // namespace cgb
