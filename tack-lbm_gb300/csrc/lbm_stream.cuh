// lbm_stream.cuh - the bulk-copy (TMA) fed AA step kernel (LBM_FLAG_BULKCOPY).
//
// The lattice is cut into row segments: SW consecutive cells of one x-row
// (y, z). A persistent CTA of SW threads walks its share of segments. For each
// segment one thread issues, per population slot, a cp.async.bulk copy of the
// contiguous row piece the segment's cells read (with a 16-byte halo on the
// side a +-x shift needs) into shared memory; an mbarrier counts the bytes.
// The cells are then updated in place in shared memory: in the AA scheme the
// post-collision population p of a cell goes exactly where the input of
// population opp(p) of the same cell came from, so each thread only touches
// its own elements. The same row pieces are then bulk-stored back to HBM.
// Three stages keep two segments' copies in flight while one is computed;
// the copies occupy no registers, so the bytes in flight per SM do not depend
// on occupancy.
//
// Only the elements a segment owns are written back: on an odd step the row
// pieces of x-shifted slots are offset by one cell, so their aligned middle
// goes back by bulk copy and the few ragged edge elements by plain stores.
// Halo elements that belong to a neighbouring segment are read but never used.
//
// Walls: free-slip rows and the lid row only change which row and slot a
// population's piece comes from (and, for the lid, adds the moving-wall term),
// uniformly for the whole segment. Segments within reach of the obstacle carry
// a per-cell link mask (bit q: population q bounces back, bit 19: obstacle
// cell); a bounce-back input is fetched with one plain load from where the
// cell parked it on the previous step (lbm_device.cuh explains the parking).
#pragma once

#include "lbm_device.cuh"

namespace lbmk {

constexpr int SW = 256;  // cells per segment = threads per CTA
constexpr long long WAIT_LIMIT = 1ll << 20;  // default mbarrier polls before a step gives up

// Bits of StreamArgs::error.
constexpr unsigned int STREAM_GAVE_UP = 1u;     // a wait ran out: the step's populations are invalid
constexpr unsigned int STREAM_IN_FLIGHT = 2u;   // a CTA ended with copies into its shared memory unconfirmed

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}
__device__ __forceinline__ void bulk_store(void *dst, const void *src, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_addr(src)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read_1() { asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

template <typename S>
struct StreamArgs {
  StepArgs<S> a;
  int nseg_x;               // segments per x-row
  int nseg;                 // segments in the lattice
  const int *seg_mask;      // per segment: first mask word, or -1 (no obstacle within reach)
  const uint32_t *masks;    // link masks, SW words per masked segment
  unsigned int *error;      // STREAM_* bits after a wait gave up
  long long wait_limit;     // mbarrier polls before a wait gives up
  int starve;               // test hook: the producer issues no copies, so every consumer wait runs out
};

// One segment: row (y, z), cells [x0, x0 + w), first link-mask word (or -1).
struct SegInfo {
  int y, z, x0, w, mslot;
};

template <typename S>
__device__ __forceinline__ SegInfo decode_seg(const StreamArgs<S> &sa, int seg) {
  SegInfo g;
  const int sx = seg % sa.nseg_x;
  const int row = seg / sa.nseg_x;
  g.y = row % sa.a.ny;
  g.z = row / sa.a.ny;
  g.x0 = sx * SW;
  g.w = min(SW, sa.a.nx - g.x0);
  g.mslot = sa.seg_mask[seg];
  return g;
}

// Direction table for lane-parallel copy issue: lane q handles population q.
struct DirTab {
  signed char cx, cy, cz, s00, s01, s10, s11, pad;
};

__device__ __forceinline__ void fill_dirtab(DirTab *tab, int tid) {
  static_for<Q>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    if (tid == q) {
      DirTab t;
      t.cx = (signed char)cx(q);
      t.cy = (signed char)cy(q);
      t.cz = (signed char)cz(q);
      t.s00 = (signed char)opp(q);
      t.s01 = (signed char)opp(dir(cx(q), cy(q), -cz(q)));
      t.s10 = (signed char)opp(dir(cx(q), -cy(q), cz(q)));
      t.s11 = (signed char)opp(dir(cx(q), -cy(q), -cz(q)));
      t.pad = 0;
      tab[q] = t;
    }
  });
}

// Where population q's row piece lives for a segment: slot, row, x-shift.
struct Piece {
  int slot, ys, zs, shift;
};

template <bool ODD, typename S>
__device__ __forceinline__ Piece piece(const StepArgs<S> &a, const DirTab &t, int q, int y, int z) {
  Piece p;
  p.slot = q;
  p.ys = y;
  p.zs = z;
  p.shift = 0;
  if (!ODD) return p;
  int ys = y - t.cy, zs = z - t.cz;
  bool ry = false, rz = false, lid = false;
  if (a.lateral == SIDE_PERIODIC) {
    ys += ys < 0 ? a.ny : 0;
    ys -= ys >= a.ny ? a.ny : 0;
  } else {
    const bool lo = ys < 0, hi = ys >= a.ny;
    lid = hi && a.lateral == SIDE_LID;
    ry = lo || (hi && a.lateral == SIDE_SLIP);
    ys = (ry || lid) ? y : ys;
  }
  if (a.vertical == SIDE_PERIODIC) {
    zs += zs < 0 ? a.nz : 0;
    zs -= zs >= a.nz ? a.nz : 0;
  } else {
    rz = zs < 0 || zs >= a.nz;
    zs = rz ? z : zs;
  }
  // the lid bounces population q back into the cell itself: its own slot q, unshifted
  if (lid) return p;
  p.slot = ry ? (rz ? t.s11 : t.s10) : (rz ? t.s01 : t.s00);
  p.ys = ys;
  p.zs = zs;
  p.shift = -t.cx;
  return p;
}

template <typename S>
struct Layout {
  static constexpr int H = 16 / (int)sizeof(S);        // halo: one 16-byte vector
  static constexpr int BUF = SW + 2 * H;               // elements per row-piece buffer
  static constexpr int STAGE = Q * BUF;                // elements per stage
  static constexpr int NST = sizeof(S) == 8 ? 4 : 5;   // pipeline stages (two CTAs per SM fit below FP64)
  static constexpr size_t BYTES = (size_t)NST * STAGE * sizeof(S) + 2 * NST * sizeof(uint64_t);
};

// The producer warp issues one segment's copies into one stage: lane q copies
// population q's row piece (one or two bulk copies) and signals `full`.
template <typename S, bool ODD>
__device__ __forceinline__ void issue_loads(const StreamArgs<S> &sa, const DirTab *tab, int seg, S *stage,
                                            uint64_t *full, SegInfo *info, int lane) {
  using L = Layout<S>;
  const StepArgs<S> &a = sa.a;
  const SegInfo g = decode_seg(sa, seg);
  if (lane == 0) *info = g;
  if (sa.starve) return;  // no arrival and no copy: the stage's `full` phase never completes
  Piece p{0, 0, 0, 0};
  uint32_t bytes = 0;
  if (lane < Q) {
    p = piece<ODD>(a, tab[lane], lane, g.y, g.z);
    bytes = (uint32_t)((g.w + (p.shift != 0 ? L::H : 0)) * sizeof(S));
  }
  const uint32_t total = __reduce_add_sync(0xffffffffu, bytes);
  if (lane == 0) mbar_arrive_expect_tx(full, total);
  __syncwarp();
  if (lane >= Q) return;
  const S *row = a.slot[p.slot] + ((size_t)p.zs * a.ny + p.ys) * a.nx;
  S *buf = stage + lane * L::BUF;
  if (p.shift == 0) {
    bulk_load(buf + L::H, row + g.x0, g.w * sizeof(S), full);
  } else if (p.shift < 0) {
    // cells read x-1: elements [x0-1, x0+w-1); load [x0-H, x0+w)
    if (g.x0 == 0) {
      bulk_load(buf, row + a.nx - L::H, L::H * sizeof(S), full);
      bulk_load(buf + L::H, row, g.w * sizeof(S), full);
    } else {
      bulk_load(buf, row + g.x0 - L::H, (g.w + L::H) * sizeof(S), full);
    }
  } else {
    // cells read x+1: elements [x0+1, x0+w+1); load [x0, x0+w+H)
    if (g.x0 + g.w == a.nx) {
      bulk_load(buf + L::H, row + g.x0, g.w * sizeof(S), full);
      bulk_load(buf + L::H + g.w, row, L::H * sizeof(S), full);
    } else {
      bulk_load(buf + L::H, row + g.x0, (g.w + L::H) * sizeof(S), full);
    }
  }
}

// The producer warp bulk-stores the aligned middle of every row piece the segment owns.
template <typename S, bool ODD>
__device__ __forceinline__ void issue_stores(const StreamArgs<S> &sa, const DirTab *tab, const SegInfo &g,
                                             S *stage, int lane) {
  using L = Layout<S>;
  if (lane >= Q) return;
  const StepArgs<S> &a = sa.a;
  const Piece p = piece<ODD>(a, tab[lane], lane, g.y, g.z);
  S *row = a.slot[p.slot] + ((size_t)p.zs * a.ny + p.ys) * a.nx;
  S *buf = stage + lane * L::BUF;
  if (p.shift == 0) bulk_store(row + g.x0, buf + L::H, g.w * sizeof(S));
  else if (p.shift < 0) bulk_store(row + g.x0, buf + L::H, (g.w - L::H) * sizeof(S));
  else bulk_store(row + g.x0 + L::H, buf + 2 * L::H, (g.w - L::H) * sizeof(S));
  bulk_commit();
}

// The ragged edge elements of x-shifted pieces: thread t < Q*H stores one.
template <typename S, bool ODD>
__device__ __forceinline__ void edge_stores(const StreamArgs<S> &sa, const DirTab *tab, const SegInfo &g,
                                            const S *stage, int t) {
  using L = Layout<S>;
  if (!ODD || t >= Q * L::H) return;
  const StepArgs<S> &a = sa.a;
  const int q = t / L::H, k = t % L::H;
  const Piece p = piece<ODD>(a, tab[q], q, g.y, g.z);
  if (p.shift == 0) return;
  S *row = a.slot[p.slot] + ((size_t)p.zs * a.ny + p.ys) * a.nx;
  const S *buf = stage + q * L::BUF;
  int e, si;  // element index in the row, index in the buffer
  if (p.shift < 0) {
    // owned: {x0-1} and [x0+w-H, x0+w-1)
    if (k == 0) {
      e = g.x0 == 0 ? a.nx - 1 : g.x0 - 1;
      si = L::H - 1;
    } else {
      e = g.x0 + g.w - L::H + k - 1;
      si = g.w + k - 1;
    }
  } else {
    // owned: [x0+1, x0+H) and {x0+w}
    if (k < L::H - 1) {
      e = g.x0 + 1 + k;
      si = L::H + 1 + k;
    } else {
      e = g.x0 + g.w == a.nx ? 0 : g.x0 + g.w;
      si = L::H + g.w;
    }
  }
  row[e] = buf[si];
}

// The one-cell update, reading and writing the stage buffers in place.
// PLAIN: no obstacle cell within reach and not the lid row.
template <typename S, int COLL, bool REPORT, bool ODD, bool PLAIN>
__device__ __forceinline__ void stream_cell(const StepArgs<S> &a, const SegInfo &g, S *stage, int i,
                                            bool lid_row, uint32_t m, float v[NSUM]) {
  using T = typename Store<S>::T;
  using L = Layout<S>;
  const bool here = !PLAIN && (m & MASK_SOLID) != 0;
  if (here && !REPORT) return;
  const int x = g.x0 + i;
  const int idx = (g.z * a.ny + g.y) * a.nx + x;
  Prev prev{0.f, 0.f, 0.f, 0.f};
  if (REPORT) prev = load_prev(a.fld, idx);
  // buffer element of population q for this cell (the lid row's y-bounced pieces are unshifted)
  auto pos = [&](auto qc) {
    constexpr int q = decltype(qc)::value;
    if (!ODD || cx(q) == 0) return q * L::BUF + L::H + i;
    if (!PLAIN && cy(q) == -1 && lid_row) return q * L::BUF + L::H + i;
    return q * L::BUF + L::H + i - cx(q);
  };
  T d[Q];
  float mx = 0.f, my = 0.f, mz = 0.f;
  static_for<Q>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    T val;
    if (PLAIN || !((m >> q) & 1u)) {
      val = Store<S>::template load<q>(stage + pos(qc));
    } else {
      const Link<S> k = make_link<S, q>(a, x, g.y, g.z);
      const T wall_term = T(6) * T(wq(q)) * k.cu;
      if (here) {
        val = rest_value<T, Store<S>::DEV>(q) + wall_term;
      } else {
        // parked on the previous step: own slot q (odd step) or the obstacle cell's slot (even)
        const T got = Store<S>::template load<q>(ODD ? a.slot[q] + idx : k.L);
        val = got + wall_term;
        const float hit = (float)(T(2) * (got + (Store<S>::DEV ? T(wq(q)) : T(0))) + wall_term);
        mx += hit * (float)(-cx(q));
        my += hit * (float)(-cy(q));
        mz += hit * (float)(-cz(q));
      }
    }
    if (!PLAIN && cy(q) == -1 && lid_row) {
      // moving lid above the top row: the cell's own population comes back with the wall term
      const T lid_term = T(6) * T(wq(q)) * (T(cx(q)) * a.u_lid);
      val = here ? rest_value<T, Store<S>::DEV>(q) + lid_term : val + lid_term;
    }
    d[q] = val;
  });
  constexpr bool DEV = Store<S>::DEV;
  Pairs<T> pr;
  const Moments<T> mo = moments<T, DEV>(d, !here, pr);
  if (!here) {
    collide<T, COLL, DEV>(d, mo, pr, a.omega_bgk, a.tau0, a.smag_c, a.magic);
    const T t = fmax(T(0), (T(x) - a.sponge_start) * a.inv_sponge_len);
    const T sigma = a.sponge_strength * t * t;
    if (sigma != T(0)) sponge<T, DEV>(d, mo, sigma, a.u0);
    static_for<Q>([&](auto pc) {
      constexpr int p = decltype(pc)::value;
      // output p goes where input opp(p) came from
      Store<S>::template store<p>(stage + pos(std::integral_constant<int, opp(p)>{}), d[p]);
    });
  }
  if (REPORT) diagnostics<T>(a.fld, idx, mo, mx, my, mz, prev, v);
}

__device__ __forceinline__ bool wait_phase(uint64_t *bar, uint32_t parity, long long limit) {
  long long polls = 0;
  while (!mbar_try_wait(bar, parity))
    if (++polls > limit) return false;
  return true;
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void consumer_sync() {
  asm volatile("bar.sync 1, %0;" ::"n"(SW) : "memory");
}

// SW consumer threads (one cell each) plus one producer warp that owns the copies.
// Stage s: `full` completes when the segment's bytes landed, `empty` when all
// consumer warps are done with it (their updates fenced for the bulk stores).
template <typename S, int COLL, bool REPORT, bool ODD>
__global__ void __launch_bounds__(SW + 32) stream_kernel(const __grid_constant__ StreamArgs<S> sa) {
  using L = Layout<S>;
  constexpr int NST = L::NST;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  S *stages = reinterpret_cast<S *>(smem_raw);
  uint64_t *full = reinterpret_cast<uint64_t *>(smem_raw + (size_t)NST * L::STAGE * sizeof(S));
  uint64_t *empty = full + NST;
  __shared__ CSum red[SW / 32][NSUM];
  __shared__ DirTab tab[Q];
  __shared__ SegInfo info[L::NST];
  __shared__ volatile int gave_up;  // a consumer's wait ran out: the producer issues nothing more
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  // this CTA's segments: blockIdx.x, blockIdx.x + gridDim.x, ...
  const int first = blockIdx.x, stride = gridDim.x;
  const int count = first < sa.nseg ? (sa.nseg - 1 - first) / stride + 1 : 0;
  fill_dirtab(tab, tid);
  if (tid == 0) {
    gave_up = 0;
    for (int s = 0; s < NST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], SW / 32);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    fence_async_smem();
  }
  __syncthreads();

  if (warp == SW / 32) {
    // producer warp: NST-1 segments ahead; a stage is refilled one iteration
    // after its stores were issued, so they have drained by then
    int issued = 0;  // segments [0, issued) have had their loads issued
    for (int k = 0; k < NST - 1 && k < count; ++k) {
      issue_loads<S, ODD>(sa, tab, first + k * stride, stages + k * L::STAGE, &full[k], &info[k], lane);
      issued = sa.starve ? 0 : k + 1;
    }
    int it = 0;
    for (; it < count; ++it) {
      const int st = it % NST;
      if (!__all_sync(0xffffffffu, wait_phase(&empty[st], (uint32_t)((it / NST) & 1), sa.wait_limit))) {
        if (lane == 0) atomicOr(sa.error, STREAM_GAVE_UP);
        break;
      }
      // the consumers' arrival for segment it carries their gave_up store
      if (gave_up) break;
      issue_stores<S, ODD>(sa, tab, info[st], stages + st * L::STAGE, lane);
      const int nxt = it + NST - 1;
      if (nxt < count) {
        const int ns = nxt % NST;  // the stage of segment it-1 (or never used yet)
        bulk_wait_read_1();        // this lane's stores of segment it-1 have read their buffer
        __syncwarp();
        issue_loads<S, ODD>(sa, tab, first + nxt * stride, stages + ns * L::STAGE, &full[ns], &info[ns], lane);
        if (!sa.starve) issued = nxt + 1;
      }
    }
    // Given up: segments it .. issued-1 may still have loads landing in this
    // CTA's shared memory (each in its own stage, one phase each, since no
    // stage was refilled before its consumers were done). Wait for them,
    // within the limit, before the CTA ends; the stages of segments before
    // `it` were all confirmed by the consumers.
    for (int j = it; j < issued; ++j)
      if (!wait_phase(&full[j % NST], (uint32_t)((j / NST) & 1), sa.wait_limit) && lane == 0)
        atomicOr(sa.error, STREAM_IN_FLIGHT);
    bulk_wait_all();
    return;
  }

  // consumer warps
  CSum acc[NSUM];
#pragma unroll
  for (int k = 0; k < NSUM; ++k) acc[k] = {0.f, 0.f};
  bool bad = false;
  for (int it = 0; it < count; ++it) {
    const int st = it % NST;
    S *stage = stages + st * L::STAGE;
    // After a wait gave up, the error is flagged, the producer is told to
    // issue nothing more, and this thread passes the remaining segments
    // through without waiting or touching memory: every barrier is still met,
    // nothing hangs.
    if (!bad && !wait_phase(&full[st], (uint32_t)((it / NST) & 1), sa.wait_limit)) {
      atomicOr(sa.error, STREAM_GAVE_UP);
      gave_up = 1;
      bad = true;
    }
    const SegInfo g = bad ? SegInfo{0, 0, 0, 0, -1} : info[st];
    const bool lid_row = sa.a.lateral == SIDE_LID && g.y == sa.a.ny - 1;
    float v[NSUM] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (tid < g.w) {
      if (g.mslot < 0 && !lid_row) {
        stream_cell<S, COLL, REPORT, ODD, true>(sa.a, g, stage, tid, false, 0u, v);
      } else {
        const uint32_t m = g.mslot >= 0 ? sa.masks[g.mslot + tid] : 0u;
        stream_cell<S, COLL, REPORT, ODD, false>(sa.a, g, stage, tid, lid_row, m, v);
      }
    }
    if (REPORT) {
#pragma unroll
      for (int k = 0; k < NSUM; ++k) {
        const CSum w = warp_csum(v[k]);
        if (lane == 0) acc[k] = csum_add(acc[k], w);
      }
    }
    if (ODD) {
      consumer_sync();  // the edge elements were written by other threads
      if (!bad) edge_stores<S, ODD>(sa, tab, g, stage, tid);
    }
    fence_async_smem();  // this thread's shared-memory writes, before the bulk stores read them
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[st]);  // one arrival per consumer warp
  }
  if (REPORT) {
    if (lane == 0)
      for (int k = 0; k < NSUM; ++k) red[warp][k] = acc[k];
    consumer_sync();
    if (tid < NSUM) {
      CSum s = red[0][tid];
      for (int w = 1; w < SW / 32; ++w) s = csum_add(s, red[w][tid]);
      sa.a.partials[(size_t)blockIdx.x * NSUM + tid] = make_float2(s.hi, s.lo);
    }
  }
}

// Link masks of the masked segments: bit q when population q of the cell
// streams from an obstacle cell (bounce-back), MASK_SOLID for an obstacle cell.
template <typename S>
__global__ void link_mask_kernel(const __grid_constant__ StepArgs<S> a, int nseg_x, const int *seg_list,
                                 int nlist, uint32_t *masks) {
  const int k = blockIdx.x;
  if (k >= nlist) return;
  const int seg = seg_list[k];
  const int sx = seg % nseg_x, row = seg / nseg_x;
  const int y = row % a.ny, z = row / a.ny;
  const int i = threadIdx.x, x = sx * SW + i;
  uint32_t m = 0;
  if (x < a.nx) {
    if (solid(a.geo, x, y, z)) m |= MASK_SOLID;
    static_for<Q>([&](auto qc) {
      constexpr int q = decltype(qc)::value;
      if (make_link<S, q>(a, x, y, z).wall) m |= 1u << q;
    });
  }
  masks[(size_t)k * SW + i] = m;
}

}  // namespace lbmk
