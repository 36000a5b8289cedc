// rz_shot.cu -- one CTA solves one shot end to end: forward Eikonal to
// convergence (eikonal.c:31-57), receiver picks and scaled residuals
// (calc_FA.c, calc_FA_res.c:34-72), and the adjoint field to convergence
// (eikonal_adj.c:31-51, init_travel_adj.c:22-58).
//
// Wavefront decomposition.  A directional Gauss-Seidel sweep (sweep.c:24-102,
// sweep_adj.c:25-75) updates cell (h,k) after its upstream neighbours
// (h-dx,k), (h,k-dy) and before its downstream neighbours.  The grid is cut
// into strips of 32 rows; warp g sweeps strip g (strip order reversed for
// dy<0) with lane l owning one row and lagging lane l-1 by one step, so at
// step t lane l updates sweep-local column t-l: an anti-diagonal.  The lane
// above hands its fresh value down with a shuffle, the lane below hands its
// still-old value up, and the last lane of a warp feeds the next warp through
// a small shared-memory ring guarded by release/acquire progress counters.
// Every update therefore sees exactly the neighbour values the reference's
// sequential loop sees, and the result is the reference's, bit for bit, in
// reference mode.
//
// Memory path.  The read-write field (T forward, lambda adjoint) streams
// through a per-warp ring of three 33x32 shared-memory tiles filled by TMA
// (cp.async.bulk.tensor) and written back by TMA; the extra row is the next
// strip's first row (old values).  Read-only per-cell data (slowness,
// converged traveltimes, adjoint skip bits, the linear sweeps' packed weights
// and receiver terms) are stored pre-skewed so that the 32 values one
// wavefront step needs are one 128-byte line: fully coalesced, staged through
// shared memory a group of eight steps ahead (the linear sweeps' second
// stream through registers).
#include <algorithm>
#include <mutex>

#include "rz_device.cuh"
#include "rz_internal.h"

namespace rz {

constexpr int kCheckSlots = 3;  // box slots in the ring of a fixpoint check
// lines the exact-adjoint preparation reads ahead of the step that uses them
constexpr int kPrepAhead = 4;
static_assert(kBlk % kPrepAhead == 0, "whole groups per item");

// Read-only stream staging.  A sweep step reads per-cell values that no
// shared-memory ring holds: the skewed slowness or traveltime line, and in
// the adjoint the edge-row values of lanes 0 and 31 and the skip word.  Each
// group of 8 steps finds them in the warp's stage slot, filled by cp.async
// during the previous group (loads into registers 8 steps ahead would leave
// the compiler free to issue them later than written).  The slot holds 8
// lines of 32 floats, lane 0's 8 and lane 31's 12-float window of edge
// values, and 8 skip words.
constexpr uint32_t kStageEdge = 1024, kStageMask = 1104;
constexpr uint32_t kStageSlot = 1152;
static_assert(kStageMask + 32 <= kStageSlot, "stage slot");

struct alignas(128) WarpShared {
    float ring[kRing][kSlotFloats];   // TMA tiles: 3 x 33 rows x 32 columns
    float hb[kHandoff];               // boundary row handed down by warp g-1
    unsigned char stage[kStageSlot];  // staged streams of one group of steps
    uint64_t full[kGroups];           // hand-off group written (producer -> this warp)
    uint64_t empty[kGroups];          // hand-off group consumed (this warp -> producer)
    uint64_t cbar[kCheckSlots];       // fixpoint check: box slot filled
    uint32_t cphase;                  // fixpoint check: expected parity per slot
};
static_assert(sizeof(WarpShared) % 128 == 0, "TMA destinations need 128-byte alignment");
static_assert(offsetof(WarpShared, hb) == sizeof(float) * kRing * kSlotFloats, "hb follows the ring");
static_assert(12 * 1024 <= sizeof(float) * kRing * kSlotFloats, "a ring lends 12 one-KB stage slots");
static_assert(offsetof(WarpShared, stage) == offsetof(WarpShared, hb) + sizeof(float) * kHandoff &&
                  offsetof(WarpShared, stage) % 16 == 0,
              "the stage slot follows hb, 16-byte aligned");

struct CtaShared {
    WarpShared *w;
    uint64_t *mbar;        // [W][kRing]
    double *red;           // [W] reduction scratch
    int *ctl;              // [8] broadcast words
    int *done;             // [W] sweeps each warp has completed (pipelined sweeps)
};

__host__ __device__ inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

size_t shot_kernel_smem(int W) {
    size_t o = sizeof(WarpShared) * W;
    o = align_up(o, 8) + sizeof(uint64_t) * kRing * W;
    o = align_up(o, 8) + sizeof(double) * W;
    o += sizeof(int) * 8 + sizeof(int) * W;
    return align_up(o, 128);
}

struct Warp {
    int g, l, z;
    uint32_t phase;  // expected parity per ring slot
    int err;
    WarpShared *ws, *ws_down;
    WarpShared *ws_all;  // every warp's shared block (pipelined sweeps)
    int *done;           // every warp's completed-sweep counter (pipelined sweeps)
    uint64_t *mbar;
    volatile int *abort_word;  // CTA-wide: a bounded wait gave up
};

// Sweep sequencing.  Banded (default): warp g takes the g-th strip of the
// band in sweep order and the CTA synchronises after every sweep.
// Pipelined (one band): warp g keeps strip g in every sweep, so for dy < 0
// its upstream neighbour is warp g+1; a warp starts its next sweep as soon as
// the strip it reads its halo row from has finished the current one, and
// hand-off groups are numbered across sweeps (no barrier re-arming), so the
// wavefront never drains between the four sweeps of a pass.
struct SweepSeq {
    int pipelined;
    int n;           // sweeps this warp has run in this launch
    int npos, nneg;  // of which with dy > 0 / dy < 0
    RZ_DEV void advance(int dy) {
        ++n;
        if (dy > 0) ++npos;
        else ++nneg;
    }
};

RZ_DEV int mod3(int v) { return v - 3 * (v / 3); }

template <bool B>
struct BoolTag {
    static constexpr bool value = B;
};

RZ_DEV float lds(uint32_t a) {
    float v;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(a));
    return v;
}
RZ_DEV void sts(uint32_t a, float v) { asm volatile("st.shared.f32 [%0], %1;" ::"r"(a), "f"(v)); }
RZ_DEV float4 lds4(uint32_t a) {
    float4 v;
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(a));
    return v;
}
RZ_DEV uint32_t lds_u32(uint32_t a) {
    uint32_t v;
    asm volatile("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(a));
    return v;
}
// cp.async: 16 bytes (both addresses 16-byte aligned, L2 only) or 4 bytes
RZ_DEV void cp_async16(uint32_t dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
RZ_DEV void cp_async4(uint32_t dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst), "l"(src) : "memory");
}
RZ_DEV void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
RZ_DEV void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

RZ_DEV unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// per-shot timeline (ns): 0 start, 1 forward done (refinement included),
// 2 residuals done, 3 adjoint prep done, 4 adjoint done, 5 first forward
// sweep done, 6 first adjoint sweep done, 7 refinement started
RZ_DEV void stamp(const ShotParams &P, int z, int slot) {
    if (P.timeline && threadIdx.x == 0) P.timeline[(size_t)z * kTimelineSlots + slot] = global_ns();
}

RZ_DEV void ring_wait(Warp &w, int slot) {
    uint32_t par = (w.phase >> slot) & 1u;
    if (!mbar_wait_copy(smem_u32(&w.mbar[slot]), par)) w.err |= ERR_TMA_TIMEOUT;
    w.phase ^= 1u << slot;
}

// ---------------------------------------------------------------------------
// one directional sweep of one warp over its strip
//   ADJ=false: forward Godunov sweep of T      (sweep.c)
//   ADJ=true : adjoint Leung-Qian sweep of lam (sweep_adj.c)
//
// Step t of the warp: lane l updates sweep-local column up = t - l of its row.
// Shared layout during a sweep: a ring of three slots, each a 33-row x
// 32-column tile (the strip's rows and its halo row) of one block, in sweep
// order.  Lane 0 fills a slot with one tile copy and drains the strip's 32
// rows with one tile store; a lane's next cell is its current cell +-4 bytes,
// or the same row of the next slot at a block boundary.
// ---------------------------------------------------------------------------
constexpr uint32_t kTileRowBytes = kBlk * 4;                  // 128
constexpr uint32_t kSlotBytes = kSlotFloats * 4;              // 4224
constexpr uint32_t kRingBytes = kRing * kSlotBytes;           // 12672

// DIV: reference-mode adjoint only, whether the verified Markstein division by
// DH may be used (P.div_fast); a compile-time choice keeps the unused
// division path out of the step code
template <int DX, int DY, bool ADJ, int MODE, int DIV = 1, bool RQS = false>
__device__ __noinline__ void sweep(const ShotParams &P, Warp &w, const CUtensorMap *mld, const CUtensorMap *mst,
                                   float &acc, uint32_t &moved, int band, int W, const SweepSeq &seq) {
    // linear sweeps over weight streams: the exact discrete adjoint, mu = R +
    // the weights neighbours put on this cell; the traveltime refinement (TAN),
    // delta = r + this cell's weights on its upwind neighbours
    constexpr bool TAN = ADJ && (MODE == kModeTangent);
    constexpr bool EX = ADJ && (MODE == kModeExact || MODE == kModeTangent);
    const int l = w.l, g = w.g;
    if (g >= W) return;  // warps beyond this grid's W only join the CTA's barriers
    const bool pipe = seq.pipelined != 0;
    const uint32_t spin = P.spin ? P.spin : kSpinLimit;  // polls before a wait for another warp gives up
    // strips are swept in bands of W (one strip per warp); sig is the strip's
    // position in sweep order, s its index from the top of the grid
    const int sig = pipe ? (DY > 0 ? g : P.nstrips - 1 - g) : band * W + g;
    if (sig >= P.nstrips) return;
    const int z = w.z;
    const int s = DY > 0 ? sig : P.nstrips - 1 - sig;
    const int j = DY > 0 ? l : 31 - l;
    const int row = kStrip * s + j;
    const bool rowok = row < P.ny;
    const int boxrow = DY > 0 ? l : 32 - l;
    const int halorow = DY > 0 ? 32 : 0;
    const bool hasUp = DY > 0 ? (row > 0) : (row < P.ny - 1);
    const bool hasDn = DY > 0 ? (row < P.ny - 1) : (row > 0);
    const int nxb = P.nxb, ncol = kBlk * nxb, nx = P.nx;
    const bool is_producer_warp = pipe ? (sig + 1 < P.nstrips) : (g + 1 < W) && (sig + 1 < P.nstrips);
    const bool is_consumer_warp = pipe ? (sig > 0) : (g > 0);
    // the warp whose strip follows in sweep order, and the hand-off groups
    // already delivered into its ring and into ours (pipelined numbering)
    WarpShared *const down = !is_producer_warp ? w.ws : pipe ? w.ws_all + (DY > 0 ? g + 1 : g - 1) : w.ws_down;
    auto delivered = [&](int strip) {  // ring of a strip receives in dy>0 sweeps unless first, dy<0 unless last
        return (strip > 0 ? seq.npos : 0) + (strip < P.nstrips - 1 ? seq.nneg : 0);
    };
    const int ngrp0 = (kBlk * P.nxb) >> 3;
    const int cons_base = pipe ? ngrp0 * delivered(s) : 0;
    const int prod_base = pipe && is_producer_warp ? ngrp0 * delivered(DY > 0 ? s + 1 : s - 1) : 0;
    const int cb8 = 8 * cons_base, pb8 = 8 * prod_base;
    if (pipe && is_producer_warp) {
        // the halo row belongs to the next strip in sweep order: it must hold
        // that strip's values after the previous sweep
        if (l == 0 && !wait_flag_ge(w.done + (DY > 0 ? g + 1 : g - 1), seq.n, w.abort_word, spin))
            w.err |= ERR_FLAG_TIMEOUT;
        __syncwarp();
        fence_proxy_async_global();
    }
    // the first warp of a later band reads its upstream row (final for this
    // sweep: the previous band is complete) from global memory
    const bool reads_prev_band = (g == 0) && (band > 0);
    const float *prev_row = nullptr;
    if (reads_prev_band) {
        const int rup = DY > 0 ? kStrip * s - 1 : kStrip * s + kStrip;
        prev_row = (ADJ ? P.L : P.T) + (size_t)z * P.fstride + (size_t)rup * P.nxp;
    }
    const bool producer = (l == 31) && is_producer_warp;
    // test hook: warp 0 withholds the signal of hand-off group 2 of its first sweep
    const bool withhold = P.withhold && g == 0 && seq.n == 0;
    const int ngrp = ncol >> 3;  // hand-off groups per sweep
    float *ring = &w.ws->ring[0][0];
    const uint32_t ring_s = smem_u32(ring);
    const uint32_t ring_end = ring_s + kRingBytes;
    const uint32_t row_off = (uint32_t)boxrow * kTileRowBytes;  // this lane's row in a tile
    const int hoff = (halorow - boxrow) * (int)kTileRowBytes;
    // tile rows: the strip's rows and the halo row, from grid row y_tile
    const int y_tile = DY > 0 ? kStrip * s : kStrip * s - 1;
    const uint32_t store_off = DY > 0 ? 0u : kTileRowBytes;  // the strip's 32 rows within a tile
    const uint32_t hb_in = smem_u32(w.ws->hb);
    const uint32_t hb_out = smem_u32(down->hb);
    const float dh = P.dh;
    const float dh_rcp = P.dh_rcp, eps_adj = P.eps_adj;
    const float eps_h2 = lq_eps_h2(eps_adj, dh);  // fast-mode Leung-Qian threshold
    constexpr bool div_fast = DIV != 0;
    // valid sweep-local columns [lo, hi) of this lane's row
    const int lo = DX > 0 ? 0 : ncol - nx;
    const int hi = rowok ? (DX > 0 ? nx : ncol) : lo;
    const bool rows_in = kStrip * s + kStrip <= P.ny;  // every row of the strip inside the grid
    const int hi_in = DX > 0 ? nx : ncol;               // hi of the rows inside the grid
    // everything the step loop touches lives in registers: shared-window
    // addresses of the barriers, the phase bits, the error bits
    const uint32_t abort_s = smem_u32((const void *)w.abort_word);
    const uint32_t mbar_s = smem_u32(w.mbar);
    const uint32_t full_in = smem_u32(w.ws->full), empty_in = smem_u32(w.ws->empty);
    const uint32_t full_out = smem_u32(down->full);
    const uint32_t empty_out = smem_u32(down->empty);
    uint32_t phase = w.phase;
    int err = 0;
    float acc_l = 0.f;  // sum of the changes (the stopping rule; the caller's acc lives in local memory)
    uint32_t moved_l = 0;  // linear sweeps: this lane moved a cell by more than 1e-6 of its value
    auto ring_wait_l = [&](int slot) {
        if (!mbar_wait_copy(mbar_s + 8u * slot, (phase >> slot) & 1u)) err |= ERR_TMA_TIMEOUT;
        phase ^= 1u << slot;
    };

    // the slot of sweep-local block k
    auto slot_base = [&](int k) -> uint32_t { return ring_s + (uint32_t)mod3(k) * kSlotBytes; };
    auto gblk = [&](int k) { return DX > 0 ? k : nxb - 1 - k; };
    // lane 0: TMA-load block k (33 rows x 32 columns) into its slot
    auto issue = [&](int k) {
        const uint32_t bar = mbar_s + 8u * (uint32_t)mod3(k);
        __syncwarp();
        if (l == 0) {
            mbar_arrive_expect_tx_a(bar, kSlotBytes);
            tma_load_3d_a(slot_base(k), mld, kBlk * gblk(k), y_tile, z, bar);
        }
    };

    // read-only per-cell streams, skewed so one step reads one 128-byte line
    constexpr bool famA = (DX == DY);
    constexpr int QS = DX > 0 ? 1 : -1;  // line step per wavefront step
    constexpr int QOFF = ADJ ? 1 : 0;    // the adjoint streams the downstream traveltime
    const float *xs;
    const uint32_t *mk = nullptr;
    const float *rs = nullptr;  // linear sweeps: own-cell R (the x stream holds packed weights, one column ahead)
    const float *ewin0 = nullptr, *ewin31 = nullptr;  // adjoint: edge values of group 0 for lanes 0 / 31
    {
        const int q0 = (DX > 0 ? 0 : ncol + 30) + QS * QOFF + kSkewFront;
        if (!ADJ) {
            xs = (famA ? P.SA : P.SB) + ((size_t)s * P.qn + q0) * 32 + j;
        } else {
            xs = (famA ? P.TA : P.TB) + (size_t)z * P.sstride + ((size_t)s * P.qn + q0) * 32 + j;
            if (EX) rs = (famA ? P.RA : P.RB) + (size_t)z * P.sstride + ((size_t)s * P.qn + (q0 - QS)) * 32 + j;
            mk = (famA ? P.MA : P.MB) + (size_t)s * P.qn + (q0 - QS * QOFF);
            // lane 0 takes its north neighbour's (dy > 0) traveltime and lambda
            // from the row above the strip, lane 31 its south one's from the row
            // below.  At step t lane 0 needs column t (dx > 0) or ncol-1-t of its
            // row, lane 31 column t-31 or ncol+30-t of its own: group G reads
            // windows of 8 and 12 floats, 16-byte aligned
            const size_t eo = (size_t)z * P.estride + (size_t)s * edge_row(P.nxp) + kEdgePad;
            const float *row0 = (DY > 0 ? P.EU : P.ED) + eo, *row31 = (DY > 0 ? P.ED : P.EU) + eo;
            ewin0 = DX > 0 ? row0 : row0 + (ncol - 8);
            ewin31 = DX > 0 ? row31 - 32 : row31 + (ncol + 20);
        }
    }
    // staging (see kStageSlot): the values of group G of 8 steps are copied
    // into the stage slot while group G-1 runs; every copy lies inside the
    // padded stream it reads (lines 0 .. 32*nxb+31 of the sweep)
    const uint32_t sg = smem_u32(w.ws->stage);
    const int ngroups = 4 * (nxb + 1);
    // the last sweep of a pass ((+x,-y) forward, (-x,-y) Leung-Qian adjoint)
    // votes per group of 8 steps whether it changed a cell of the strip
    constexpr bool REC = !EX && (ADJ ? (DX < 0 && DY < 0) : (DX > 0 && DY < 0));
    uint8_t *const chg = (REC && P.chg) ? P.chg + (size_t)z * P.chg_stride + (size_t)s * ngroups : nullptr;
    const float *xline = xs - j;  // the 32-float line of step 0
    // RQS (linear sweeps): the second stream (receiver terms or residuals) is
    // staged like the first, group by group, in a 1 KB slot that a warp which
    // does not sweep lends from its ring (warp W + g/12, slot g%12; its
    // barriers are not touched, and no phase that uses that ring overlaps the
    // sweeps).  Without RQS the stream is read through registers 8 steps
    // ahead, which leaves the loads' latency exposed (the exact adjoint's
    // sweeps run 25% longer).  sweep_dispatch chooses.
    constexpr bool RQ = EX && RQS;
    const uint32_t sq = RQ ? smem_u32(&w.ws_all[W + g / 12].ring[0][0]) + 1024u * (uint32_t)(g % 12) : 0u;
    const float *rline = RQ ? rs - j : nullptr;
    auto stage_issue = [&](int G) {
        const uint32_t dst = sg;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int c = l + 32 * h, line = c >> 3, piece = c & 7;
            cp_async16(dst + 16u * (uint32_t)c, xline + QS * 32 * (8 * G + line) + 4 * piece);
        }
        if (ADJ && l < 2) cp_async16(dst + kStageEdge + 16u * (uint32_t)l, ewin0 + (DX > 0 ? 8 * G : -8 * G) + 4 * l);
        if (ADJ && l >= 2 && l < 5)
            cp_async16(dst + kStageEdge + 16u * (uint32_t)l, ewin31 + (DX > 0 ? 8 * G : -8 * G) + 4 * (l - 2));
        if (ADJ && !EX && l < 8) cp_async4(dst + kStageMask + 4u * (uint32_t)l, mk + QS * (8 * G + l));
        if (RQ) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int c = l + 32 * h, line = c >> 3, piece = c & 7;
                cp_async16(sq + 16u * (uint32_t)c, rline + QS * 32 * (8 * G + line) + 4 * piece);
            }
        }
        cp_async_commit();
    };

    float xq[8];
    uint32_t mq[8];
    float eq[8];
    float rq[8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
        if (EX && !RQ) rq[i] = __ldca(rs + QS * 32 * i);
    stage_issue(0);
    float c_tt = 0.f, w_tt = 0.f;  // exact adjoint: x weights of this and the previous column
    float c_wz = 0.f, w_wz = 0.f;  // exact adjoint: z weights of this and the previous column
    if (ADJ && !EX) c_tt = __ldca(xs - QS * 32);
    if (EX) unpack_weights(__ldca(xs - QS * 32), c_tt, c_wz);

    issue(0);
    if (nxb > 1) issue(1);
    ring_wait_l(0);

    // ring address of this lane's cell at step t = 0 (column up = -l, which
    // for l > 0 lies before the sweep: any ring cell serves, nothing reads it)
    auto advance = [&](uint32_t a) -> uint32_t {
        // (a - ring_s) % 128 is 4 * (column in the block): tiles and rows are 128-byte multiples
        if (DX > 0) {
            a += 4;
            if ((a & (kTileRowBytes - 1)) == 0) {  // past column 31: column 0 of the next slot
                a += kSlotBytes - kTileRowBytes;
                if (a >= ring_end) a -= kRingBytes;
            }
            return a;
        } else {
            if ((a & (kTileRowBytes - 1)) == 0) {  // at column 0: column 31 of the next slot
                a += kSlotBytes + kTileRowBytes - 4;
                return a >= ring_end ? a - kRingBytes : a;
            }
            return a - 4;
        }
    };
    // the inverse of advance
    auto retreat = [&](uint32_t a) -> uint32_t {
        if (DX > 0) {
            if ((a & (kTileRowBytes - 1)) == 0) {  // at column 0: column 31 of the previous slot
                a = a < ring_s + kSlotBytes ? a + kRingBytes : a;
                return a - kSlotBytes + kTileRowBytes - 4;
            }
            return a - 4;
        } else {
            a += 4;
            if ((a & (kTileRowBytes - 1)) == 0) {  // past column 31: column 0 of the previous slot
                a -= kTileRowBytes;
                a = a < ring_s + kSlotBytes ? a + kRingBytes : a;
                a -= kSlotBytes;
            }
            return a;
        }
    };
    static_assert((kSlotBytes % kTileRowBytes) == 0 && (kTileRowBytes & (kTileRowBytes - 1)) == 0, "tile layout");
    uint32_t addr_c = slot_base(0) + row_off + (DX > 0 ? 0u : 31u * 4u);
    for (int q = 0; q < l; ++q) addr_c = retreat(addr_c);
    uint32_t addr_e = advance(addr_c);
    float own_next = lds(addr_c);
    float ev_next = lds(addr_e);
    float halo_next = lds(addr_c + hoff);

    float res_prev = 0.f;
    float hand_carry = 0.f;  // the last step's value of the previous group (lane 31 hands it down)
    for (int k = 0; k <= nxb; ++k) {
#pragma unroll 1
        for (int i0 = 0; i0 < 32; i0 += 8) {
            const int t0 = kBlk * k + i0;
            // ---- group prologue: every wait and branch of the next 8 steps ----
            // refill: block k+1 goes where block k-2 was; its write-back, issued
            // at the end of the previous round, has had 8 steps to read shared
            // memory, and lane 0 first reads the new block at step 30
            if (i0 == 8 && k >= 1 && k + 1 < nxb) {
                // generic accesses of the slot (including writes of lanes
                // still outside the sweep) are ordered before the TMA refill
                fence_proxy_async_smem();
                tma_store_wait_read<0>();
                issue(k + 1);
            }
            if (i0 == 24 && k + 1 < nxb) ring_wait_l(mod3(k + 1));
            // boundary-row values lane 0 needs in these 8 steps (columns t0..t0+7)
            float hbq[8];
            if (is_consumer_warp) {
                const int G = t0 >> 3;
                if (G < ngrp) {
                    const int Gg = G + cons_base;  // group number in this ring's lifetime
                    if (!mbar_wait_a(full_in + 8u * (Gg & (kGroups - 1)), (Gg >> kGroupsLog2) & 1, abort_s, spin))
                        err |= ERR_FLAG_TIMEOUT;
                    const uint32_t hb_g = hb_in + 4u * (uint32_t)((t0 + cb8) & (kHandoff - 1));  // 32-byte aligned
                    const float4 h0 = lds4(hb_g), h1 = lds4(hb_g + 16u);
                    hbq[0] = h0.x, hbq[1] = h0.y, hbq[2] = h0.z, hbq[3] = h0.w;
                    hbq[4] = h1.x, hbq[5] = h1.y, hbq[6] = h1.z, hbq[7] = h1.w;
                    // the values are in registers: release the slot at once
                    mbar_arrive_if(empty_in + 8u * (Gg & (kGroups - 1)), l == 0);
                } else {
#pragma unroll
                    for (int q = 0; q < 8; ++q) hbq[q] = 0.f;
                }
            } else if (reads_prev_band) {
                // lane 0's columns t0..t0+7 of the row above the band (written by
                // TMA earlier in this launch: read through L2)
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const int uq = min(max(t0 + q, 0), ncol - 1);
                    hbq[q] = __ldcg(prev_row + (DX > 0 ? uq : ncol - 1 - uq));
                }
            } else {
#pragma unroll
                for (int q = 0; q < 8; ++q) hbq[q] = 0.f;
            }
            if (is_producer_warp) {
                // lane 31 writes hand-off group Gp (columns t0-32 .. t0-25) in this group
                const int Gp = (t0 - 32) >> 3, Gpg = Gp + prod_base;
                if (t0 >= 32 && Gpg >= kGroups && Gp < ngrp &&
                    !mbar_wait_a(empty_out + 8u * (Gpg & (kGroups - 1)), ((Gpg >> kGroupsLog2) - 1) & 1, abort_s,
                                 spin))
                    err |= ERR_FLAG_TIMEOUT;
            }
            {
                const int G = t0 >> 3;
                cp_async_wait_all();  // group G's values (copied during group G-1) have landed
                __syncwarp();         // ... for every lane
#pragma unroll
                for (int ii = 0; ii < 8; ++ii) {
                    xq[ii] = lds(sg + 128u * (uint32_t)ii + 4u * (uint32_t)j);
                    if (ADJ) {  // only lanes 0 and 31 use their edge value
                        const int ei = l == 0 ? (DX > 0 ? ii : 7 - ii) : 8 + (DX > 0 ? ii + 1 : 10 - ii);
                        eq[ii] = lds(sg + kStageEdge + 4u * (uint32_t)ei);
                    }
                    if (ADJ && !EX) mq[ii] = lds_u32(sg + kStageMask + 4u * (uint32_t)ii);
                    if (RQ) rq[ii] = lds(sq + 128u * (uint32_t)ii + 4u * (uint32_t)j);
                }
                __syncwarp();  // every lane has read the slot: refill it
                if (G + 1 < ngroups) stage_issue(G + 1);
            }
            const int u0 = t0 - l;
            const float *rr = EX ? rs + QS * 32 * t0 : nullptr;
            // ---- 8 wavefront steps, straight-line code.  In an interior group
            // (every lane's 8 columns strictly inside the grid, every row of the
            // strip inside it) no cell is a boundary cell or outside the grid
            // and every hand-off value is in range: those tests are left out.
            bool changed = false;  // REC: this lane changed a cell in this group
            auto steps8 = [&](auto interior_tag) {
                constexpr bool INT = decltype(interior_tag)::value;
                // lane 31 of a producing warp hands down the values of columns
                // upp0 .. upp0+7 (steps t0-1 .. t0+6): two 16-byte stores, then
                // the group's full barrier
                const int upp0 = t0 - 32;
                const bool hand = producer && (INT || (upp0 >= 0 && upp0 < ncol));
                const uint32_t hq = hb_out + 4u * (uint32_t)((upp0 + pb8) & (kHandoff - 1));  // 32-byte aligned
                float h0 = 0.f, h1 = 0.f, h3 = 0.f, h4 = 0.f, h5 = 0.f;
                // addr_e reaches sweep-local column t0+ii-l+2 at step ii: a new block
                // (the next slot) when that column is a multiple of 32, at most once
                // in 8 steps (at ii = cx); the jump there is advance's
                const int cx = (l - t0 - 2) & 31;
                const uint32_t m = (addr_e - ring_s) / kSlotBytes;  // slot before the crossing
                const uint32_t jump = (DX > 0 ? 4u + kSlotBytes - kTileRowBytes : kSlotBytes + kTileRowBytes - 4u) -
                                      (m == kRing - 1 ? kRingBytes : 0u);
#pragma unroll
            for (int ii = 0; ii < 8; ++ii) {
                const int up = u0 + ii;
                const float own = own_next;
                const float ev = ev_next;
                const float halo = halo_next;
                const uint32_t cur = addr_c;
                // prefetch the next step's shared values
                addr_c = addr_e;
                addr_e += (ii == cx) ? jump : (uint32_t)(DX > 0 ? 4 : -4);
                own_next = ev;
                ev_next = lds(addr_e);
                halo_next = lds(addr_c + hoff);

                float nv = __shfl_up_sync(0xffffffffu, res_prev, 1);
                float sv = __shfl_down_sync(0xffffffffu, ev, 1);
                nv = (l == 0) ? hbq[ii] : nv;
                sv = (l == 31) ? halo : sv;
                const float xv = xq[ii];
                const bool valid = INT || (unsigned)(up - lo) < (unsigned)(hi - lo);
                float r;
                if (!ADJ) {
                    const bool hasW = INT || up > lo;
                    const bool hasE = INT || up < hi - 1;
                    const float tw = hasW ? res_prev : own;
                    const float te = hasE ? ev : own;
                    const float tn = hasUp ? nv : own;
                    const float ts = hasDn ? sv : own;
                    const float a = fminf(tw, te), b = fminf(tn, ts);
                    const float tt =
                        (MODE == kModeReference) ? godunov_ref(a, b, xv, dh) : godunov_fast(a, b, xv, dh);
                    r = fminf(own, tt);
                    r = valid ? r : own;
                } else if (EX) {
                    float e_wx, e_wz;  // weights of the cell one column downstream
                    unpack_weights(xv, e_wx, e_wz);
                    const float rcell = rq[ii];
                    if (!RQ) rq[ii] = __ldca(rr + QS * 32 * (ii + 8));
                    const float edge = eq[ii];
                    float n_wz = __shfl_up_sync(0xffffffffu, w_wz, 1);
                    float s_wz = __shfl_down_sync(0xffffffffu, e_wz, 1);
                    n_wz = (l == 0) ? edge : n_wz;
                    s_wz = (l == 31) ? edge : s_wz;
                    // weights of the grid neighbours (signed: < 0 points west / north)
                    const float wxE = DX > 0 ? e_wx : w_tt, wxW = DX > 0 ? w_tt : e_wx;
                    const float wzS = DY > 0 ? s_wz : n_wz, wzN = DY > 0 ? n_wz : s_wz;
                    const float lE = DX > 0 ? ev : res_prev, lW = DX > 0 ? res_prev : ev;
                    const float lS = DY > 0 ? sv : nv, lN = DY > 0 ? nv : sv;
                    float m = rcell;
                    if (TAN) {
                        // own weights: < 0 on the west / north neighbour, > 0 on the east / south one
                        // (the other side's term adds an exact zero: no branch on the weights)
                        m = fmaf(fmaxf(c_tt, 0.f), lE, fmaf(fmaxf(-c_tt, 0.f), lW, m));
                        m = fmaf(fmaxf(c_wz, 0.f), lS, fmaf(fmaxf(-c_wz, 0.f), lN, m));
                    } else {
                        m = wxW > 0.f ? fmaf(wxW, lW, m) : m;
                        m = wxE < 0.f ? fmaf(-wxE, lE, m) : m;
                        m = wzN > 0.f ? fmaf(wzN, lN, m) : m;
                        m = wzS < 0.f ? fmaf(-wzS, lS, m) : m;
                    }
                    r = valid ? m : own;
                    w_tt = c_tt;
                    c_tt = e_wx;
                    w_wz = c_wz;
                    c_wz = e_wz;
                } else {
                    const uint32_t mword = mq[ii];
                    const float edge = eq[ii];
                    const float e_tt = xv;  // traveltime one column downstream
                    float n_tt = __shfl_up_sync(0xffffffffu, w_tt, 1);
                    float s_tt = __shfl_down_sync(0xffffffffu, e_tt, 1);
                    n_tt = (l == 0) ? edge : n_tt;
                    s_tt = (l == 31) ? edge : s_tt;
                    const float tE = DX > 0 ? e_tt : w_tt, tW = DX > 0 ? w_tt : e_tt;
                    const float tS = DY > 0 ? s_tt : n_tt, tN = DY > 0 ? n_tt : s_tt;
                    const float lE = DX > 0 ? ev : res_prev, lW = DX > 0 ? res_prev : ev;
                    const float lS = DY > 0 ? sv : nv, lN = DY > 0 ? nv : sv;
                    if (MODE == kModeReference) {
                        DivDH div{dh, dh_rcp, div_fast};
                        r = leung_qian_ref(c_tt, tE, tW, tS, tN, lE, lW, lS, lN, own, div, eps_adj);
                    } else {
                        r = leung_qian_fast(c_tt, tE, tW, tS, tN, lE, lW, lS, lN, own, eps_h2);
                    }
                    const bool keep = !valid || ((mword >> j) & 1u);
                    r = keep ? own : r;
                    w_tt = c_tt;
                    c_tt = e_tt;
                }
                sts(cur, r);
                if (MODE == kModeFast || MODE == kModeReference) acc_l += valid ? own - r : 0.0f;
                // linear sweeps: a cell moved by more than 1e-6 of its value
                if (EX) moved_l |= (uint32_t)(valid && !(fabsf(own - r) <= 1e-6f * fabsf(r)));
                if (ii == 0) h0 = r;
                if (ii == 1) h1 = r;
                if (ii == 2) sts4_if(hq, hand_carry, h0, h1, r, hand);
                if (ii == 3) h3 = r;
                if (ii == 4) h4 = r;
                if (ii == 5) h5 = r;
                if (ii == 6) {
                    sts4_if(hq + 16u, h3, h4, h5, r, hand);
                    mbar_arrive_if(full_out + 8u * (uint32_t)(((upp0 + pb8) >> 3) & (kGroups - 1)),
                                   hand && !(withhold && upp0 == 16));
                }
                if (ii == 7) hand_carry = r;
                if (REC) changed |= valid && r != own;
                res_prev = r;
            }
            };
            // the columns of this group: t0-31 (lane 31) .. t0+7 (lane 0)
            if (rows_in && t0 - 31 >= lo + 1 && t0 + 7 <= hi_in - 2) steps8(BoolTag<true>{});
            else steps8(BoolTag<false>{});
            if (REC && chg) {
                const bool any = __any_sync(0xffffffffu, changed);
                if (l == 0) chg[t0 >> 3] = any ? 1 : 0;
            }
        }
        // block k-1 is complete: lane 0 writes the strip's 32 rows back (rows
        // past the grid are clipped by the map)
        if (k >= 1) {
            fence_proxy_async_smem();
            __syncwarp();
            if (l == 0) {
                tma_store_3d_a(mst, kBlk * gblk(k - 1), kStrip * s, z, slot_base(k - 1) + store_off);
                tma_store_commit();
            }
        }
    }
    tma_store_wait_all<0>();
    fence_proxy_async_global();
    if (RQ) fence_proxy_async_smem();  // the lent slot's copies precede later tensor copies into that ring
    __syncwarp();
    if (pipe && l == 0) st_release_smem(w.done + g, seq.n + 1);
    w.phase = phase;
    w.err |= err;
    acc += acc_l;
    moved |= moved_l;
}

// ---------------------------------------------------------------------------
// CTA-wide helpers
// ---------------------------------------------------------------------------
RZ_DEV double block_sum(double v, const CtaShared &sh) {
    const int l = threadIdx.x & 31, g = threadIdx.x >> 5, W = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if (l == 0) sh.red[g] = v;
    __syncthreads();
    double t = 0.0;
    for (int i = 0; i < W; ++i) t += sh.red[i];
    __syncthreads();
    return t;
}

// (re)arm this warp's hand-off barriers; every sweep starts at group 0
RZ_DEV void handoff_init(WarpShared *ws, bool reinit) {
    if ((threadIdx.x & 31) == 0) {
        for (int i = 0; i < kGroups; ++i) {
            if (reinit) {
                mbar_inval(&ws->full[i]);
                mbar_inval(&ws->empty[i]);
            }
            mbar_init(&ws->full[i], 1);
            mbar_init(&ws->empty[i], 1);
        }
    }
}

// between sweeps: all stores done, hand-off barriers re-armed
RZ_DEV void sweep_barrier(const CtaShared &sh) {
    __syncthreads();
    handoff_init(&sh.w[threadIdx.x >> 5], true);
    __syncthreads();
}

// Reference stopping rule (norm1.c:20-29, eikonal.c:44): continue while
// mean|F-Fold| >= TTNORM, the mean being a sequential float sum in x-outer
// order.  The estimate is the pass's own change: every update is
// min(own, new), so a cell's changes over the pass's sweeps add up to
// Fold - F, and each lane summed its cells' changes (`acc`; `terms` bounds a
// lane's float additions, the per-sweep totals included).  It decides
// whenever it is certain; within the worst-case rounding window of the
// sequential sum and of the estimate the exact sequential sum is replayed
// from F and Fold (rare).  A first pass starts from the initial field, which
// is not copied: with fold_ok false, rebuild(Fold) writes it (CTA-wide)
// before a replay.
template <class Rebuild>
RZ_DEV bool ref_continue(const ShotParams &P, const float *F, float *Fold, const CtaShared &sh, float acc,
                         double terms, bool fold_ok, Rebuild &&rebuild) {
    const int n = P.nx * P.ny;
    double est = block_sum((double)acc, sh);
    if (threadIdx.x == 0) {
        int decision;  // 1 continue, 0 stop, 2 undecided
        if (est == 0.0) {
            decision = 0;
        } else {
            // each change rounded once, then added: 2 roundings per term
            double gam = ((double)n + 2.0 * terms + 4.0) * 0x1p-24 + 0x1p-20;
            double thr = (double)P.ttnorm * (double)n;
            if (est * (1.0 - gam) > thr * (1.0 + 0x1p-21)) decision = 1;
            else if (est * (1.0 + gam) < thr * (1.0 - 0x1p-21)) decision = 0;
            else decision = 2;
        }
        sh.ctl[0] = decision;
    }
    __syncthreads();
    int d = sh.ctl[0];
    __syncthreads();
    if (d == 2) {
        if (!fold_ok) {
            rebuild(Fold);
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            float sum = 0.f;
            for (int h = 0; h < P.nx; ++h)
                for (int k = 0; k < P.ny; ++k) {
                    size_t o = (size_t)k * P.nxp + h;
                    float dv = fabsf(__fsub_rn(__ldcg(F + o), __ldcg(Fold + o)));
                    sum = __double2float_rn(__dadd_rn((double)sum, (double)dv));
                }
            float l1 = __fdiv_rn(sum, __int2float_rn(n));
            sh.ctl[0] = (l1 >= P.ttnorm) ? 1 : 0;
        }
        __syncthreads();
        d = sh.ctl[0];
        __syncthreads();
    }
    return d != 0;
}

// Fixpoint checks.  Every point update of a sweep is F_c = min(own, G_c)
// of the current field; if no cell of the field would change under F (each
// evaluated on the same field, in the sweep's arithmetic), then a
// Gauss-Seidel pass changes nothing: its first update leaves the field as it
// is, hence so does the second, and so on through all four sweeps.  Such a
// pass has zero change, so the stopping rule ends the loop after it; the
// caller counts it without sweeping it, and every result stays the same.
// The checks split the grid into tasks of 128 columns x at most P.check_rows
// rows (kCheckRows by default; check_task_rows balances the tasks over the
// warps; the autotuner picks the cap).  A
// warp walks a task top to bottom, four cells per lane.  Lane 0 loads the
// task's rows in boxes of kCheckBox rows by tensor-map copies into a ring of
// three slots (one mbarrier each) in the warp's shared memory.  A box of a
// field whose east and west neighbours are needed is kCheckHaloCols wide and
// starts 4 columns west of the task (a 16-byte aligned start), so it carries
// the neighbours of the task's edge cells; cells outside the grid read as the
// fill value and are never used.  Neighbours across lanes come by shuffle.
// Boxes rather than row copies: small bulk copies are bound by the copy
// engine's instruction rate, and a box moves four rows per instruction.
constexpr int kCheckRows = 64, kCheckBox = kCheckBoxRows, kCheckHaloCols = kCheckCols;

// Rows per task for `rows` rows in nch column chunks and W warps: the fewest
// rounds of W tasks times (rows per task + one box of start-up), at most
// cap rows per task.
RZ_DEV int check_task_rows(int rows, int nch, int W, int cap) {
    const int n0 = (rows + cap - 1) / cap;
    int best_r = cap, best = 0x7fffffff;
    for (int nrb = n0; nrb <= 4 * n0 + 4; ++nrb) {
        const int r = (rows + nrb - 1) / nrb;
        const int cost = ((nch * nrb + W - 1) / W) * (r + kCheckBox);
        if (cost < best) best = cost, best_r = r;
    }
    return best_r;
}
static_assert(kCheckBox == 4 && kCheckHaloCols == 128 + 8, "box rows are indexed with j >> 2, halos are 4 columns");
constexpr uint32_t kRowH = kCheckHaloCols * 4;  // bytes of a box row with halos
constexpr uint32_t kRowP = 128 * 4;             // bytes of a box row without
constexpr uint32_t kCheckSlotF = kCheckBox * (kRowH + kRowP);  // forward: T box, slowness box
constexpr uint32_t kCheckSlotA = kCheckBox * 2 * kRowH;        // adjoint: T box, lambda box
static_assert(kCheckSlots * kCheckSlotF <= sizeof(float) * kRing * kSlotFloats, "forward check ring");
static_assert(kCheckSlots * kCheckSlotA <= offsetof(WarpShared, full),
              "adjoint check ring (hand-off row and stage slot are idle between sweeps)");
static_assert(kCheckSlotF % 128 == 0 && kCheckSlotA % 128 == 0, "box slots stay 128-byte aligned");


// four cells of a row with their west and east neighbours; the row starts
// with the 4 halo columns, lane l's cells are at 16 + 16 l
struct Row4 {
    float w, v[4], e;
};
RZ_DEV Row4 box_row4(uint32_t row, int l) {
    Row4 r;
    const float4 c = lds4(row + 16u + 16u * l);
    r.v[0] = c.x, r.v[1] = c.y, r.v[2] = c.z, r.v[3] = c.w;
    r.w = __shfl_up_sync(0xffffffffu, c.w, 1);
    r.e = __shfl_down_sync(0xffffffffu, c.x, 1);
    if (l == 0) r.w = lds(row + 12u);
    if (l == 31) r.e = lds(row + 16u + 512u);
    return r;
}

// Whether the last sweep of the pass (x direction dx) changed a cell of a
// strip touching rows [r_lo, r_hi] in a group of 8 steps whose columns meet
// [c_lo, c_hi]; true without votes.  A cell none of whose neighbours changed
// after that sweep evaluated it has the same update now, which it did not
// fall below: the checks skip a task when no vote covers the task and the
// cells around it.  Group G of a sweep covers sweep-local columns
// 8G-31 .. 8G+7 (lanes 31 .. 0).
RZ_DEV bool votes_any(const ShotParams &P, int z, int r_lo, int r_hi, int c_lo, int c_hi, int dx) {
    if (!P.chg) return true;
    const int l = threadIdx.x & 31, ng = 4 * (P.nxb + 1), ncol = kBlk * P.nxb;
    r_lo = max(r_lo, 0), r_hi = min(r_hi, P.ny - 1);
    const int s_lo = r_lo >> 5, s_hi = r_hi >> 5;
    const int u_lo = dx > 0 ? c_lo : ncol - 1 - c_hi, u_hi = dx > 0 ? c_hi : ncol - 1 - c_lo;  // sweep-local
    const int g_lo = max(0, u_lo >> 3), g_hi = min(ng - 1, (u_hi + 31) >> 3);  // 8G+7 >= u_lo, 8G-31 <= u_hi
    const int ngs = g_hi - g_lo + 1, total = (s_hi - s_lo + 1) * max(ngs, 0);
    const uint8_t *v = P.chg + (size_t)z * P.chg_stride;
    bool any = false;
    for (int i = l; i < total; i += 32) any |= v[(size_t)(s_lo + i / ngs) * ng + g_lo + i % ngs] != 0;
    return __any_sync(0xffffffffu, any);
}

// box ring of a check: box b of a task sits in slot b % kCheckSlots
struct CheckRing {
    uint32_t base, bars, abort_s, phase;
    int err;
    RZ_DEV void wait(int b) {
        const int s = b % kCheckSlots;
        if (!mbar_wait_copy(bars + 8u * s, (phase >> s) & 1u)) err |= ERR_TMA_TIMEOUT;
        phase ^= 1u << s;
    }
};

// returns 1 when no cell would change, plus the error flags shifted left by one.
// mT: traveltime fields, box kCheckHaloCols x kCheckBox; mS: slowness [ny][nxp],
// box 128 x kCheckBox; z: this shot's field.
template <int MODE>
__device__ __noinline__ int forward_is_fixpoint(const ShotParams &P, const CUtensorMap *mT, const CUtensorMap *mS,
                                                int z, WarpShared *ws, int *found, volatile int *abort_word) {
    const int nx = P.nx, ny = P.ny;
    const int l = threadIdx.x & 31, g = threadIdx.x >> 5, W = blockDim.x >> 5;
    const int cap = P.check_rows > 0 ? P.check_rows : kCheckRows;
    const int nch = (nx + 127) >> 7, rt = check_task_rows(ny, nch, W, cap), nrb = (ny + rt - 1) / rt;
    if (threadIdx.x == 0) *found = 0;
    fence_proxy_async_smem();  // the ring's generic accesses precede the copies
    __syncthreads();
    CheckRing R{smem_u32(&ws->ring[0][0]), smem_u32(ws->cbar), smem_u32((const void *)abort_word), ws->cphase, 0};
    bool change = false;
    for (int task = g; task < nch * nrb && !change; task += W) {
        if (__shfl_sync(0xffffffffu, *(volatile int *)found, 0)) break;  // warp-uniform
        const int base = (task % nch) << 7, h0 = base + 4 * l;
        // rows k0 .. k0+kk-1; window row j is grid row k0-1+j, j = 0 .. kk+1
        const int k0 = (task / nch) * rt, kk = min(ny - k0, rt);
        if (!votes_any(P, z, k0 - 1, k0 + kk, base - 1, base + 128, +1)) continue;  // (+x,-y) was last
        const int nb = ((kk + 1) >> 2) + 1;
        auto issue = [&](int b) {
            if (b >= nb || l != 0) return;
            const uint32_t sl = R.base + (uint32_t)(b % kCheckSlots) * kCheckSlotF;
            const uint32_t br = R.bars + 8u * (uint32_t)(b % kCheckSlots);
            mbar_arrive_expect_tx_a(br, kCheckSlotF);
            tma_load_3d_a(sl, mT, base - 4, k0 - 1 + kCheckBox * b, z, br);
            tma_load_3d_a(sl + kCheckBox * kRowH, mS, base, k0 - 1 + kCheckBox * b, 0, br);
        };
        auto trow = [&](int j) {
            return R.base + (uint32_t)((j >> 2) % kCheckSlots) * kCheckSlotF + (uint32_t)(j & 3) * kRowH;
        };
        issue(0), issue(1), issue(2);
        __syncwarp();
        R.wait(0);
        // interior task: every cell has all four neighbours inside the grid
        const bool interior = base > 0 && base + 128 < nx && k0 > 0 && k0 + kk < ny;
        auto rows = [&](auto interior_tag) {
            constexpr bool INT = decltype(interior_tag)::value;
        for (int b = 0; b < nb; ++b) {
#pragma unroll
            for (int r = 0; r < kCheckBox; ++r) {
                const int j = kCheckBox * b + r, k = k0 - 1 + j;
                if (j < 1 || j > kk) continue;  // warp-uniform
                if (r == kCheckBox - 1) R.wait(b + 1);  // holds row j+1
                const uint32_t rc = trow(j);
                const Row4 c = box_row4(rc, l);
                const float4 u = lds4(trow(j - 1) + 16u + 16u * l), d = lds4(trow(j + 1) + 16u + 16u * l);
                const float4 s4 = lds4(rc - (uint32_t)(j & 3) * kRowH + kCheckBox * kRowH + (uint32_t)(j & 3) * kRowP +
                                       16u * l);
                const float uv[4] = {u.x, u.y, u.z, u.w}, dv[4] = {d.x, d.y, d.z, d.w};
                const float sv[4] = {s4.x, s4.y, s4.z, s4.w};
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int h = h0 + i;
                    const float own = c.v[i];
                    const float tw = (INT || h > 0) ? (i == 0 ? c.w : c.v[i - 1]) : own;
                    const float te = (INT || h < nx - 1) ? (i == 3 ? c.e : c.v[i + 1]) : own;
                    const float tn = (INT || k > 0) ? uv[i] : own, ts = (INT || k < ny - 1) ? dv[i] : own;
                    const float a = fminf(tw, te), bb = fminf(tn, ts);
                    const float tt = (MODE == kModeReference) ? godunov_ref(a, bb, sv[i], P.dh)
                                                              : godunov_fast(a, bb, sv[i], P.dh);
                    change |= (INT || h < nx) && (tt < own);
                }
            }
            // box b-1 is read by no later row: box b+2 takes its slot
            fence_proxy_async_smem();
            __syncwarp();
            if (b >= 1) issue(b + 2);
        }
        };
        if (interior) rows(BoolTag<true>{});
        else rows(BoolTag<false>{});
        change = __any_sync(0xffffffffu, change);
        if (change && l == 0) *(volatile int *)found = 1;
    }
    if (l == 0) ws->cphase = R.phase;
    fence_proxy_async_smem();  // before the next sweep's copies into the ring
    return (__syncthreads_or(change) ? 0 : 1) | (R.err << 1);
}

// the Leung-Qian update of interior, non-receiver cells (sweep_adj.c:26-30);
// skip is the [ny][nxp] byte map of cells the adjoint sweeps leave unchanged.
// mT / mL: traveltime / lambda fields, box kCheckHaloCols x kCheckBox.
template <int MODE, int DIV>
__device__ __noinline__ int adjoint_is_fixpoint(const ShotParams &P, const CUtensorMap *mT, const CUtensorMap *mL,
                                                int z, WarpShared *ws, int *found, volatile int *abort_word) {
    const int nx = P.nx, ny = P.ny, nxp = P.nxp;
    const int l = threadIdx.x & 31, g = threadIdx.x >> 5, W = blockDim.x >> 5;
    const int cap = P.check_rows > 0 ? P.check_rows : kCheckRows;
    const int nch = (nx + 127) >> 7, rt = check_task_rows(ny - 2, nch, W, cap), nrb = (ny - 2 + rt - 1) / rt;
    const DivDH div{P.dh, P.dh_rcp, DIV != 0};
    const float eps_h2 = lq_eps_h2(P.eps_adj, P.dh);  // fast-mode Leung-Qian threshold
    if (threadIdx.x == 0) *found = 0;
    fence_proxy_async_smem();  // the ring's generic accesses precede the copies
    __syncthreads();
    CheckRing R{smem_u32(&ws->ring[0][0]), smem_u32(ws->cbar), smem_u32((const void *)abort_word), ws->cphase, 0};
    bool change = false;
    for (int task = g; task < nch * nrb && !change; task += W) {
        if (__shfl_sync(0xffffffffu, *(volatile int *)found, 0)) break;  // warp-uniform
        const int base = (task % nch) << 7, h0 = base + 4 * l;
        // interior rows k0 .. k0+kk-1 (k0 >= 1, k0+kk <= ny-1); window row j is grid row k0-1+j
        const int k0 = 1 + (task / nch) * rt, kk = min(ny - 1 - k0, rt);
        if (!votes_any(P, z, k0 - 1, k0 + kk, base - 1, base + 128, -1)) continue;  // (-x,-y) was last
        const int nb = ((kk + 1) >> 2) + 1;
        auto issue = [&](int b) {
            if (b >= nb || l != 0) return;
            const uint32_t sl = R.base + (uint32_t)(b % kCheckSlots) * kCheckSlotA;
            const uint32_t br = R.bars + 8u * (uint32_t)(b % kCheckSlots);
            mbar_arrive_expect_tx_a(br, kCheckSlotA);
            tma_load_3d_a(sl, mT, base - 4, k0 - 1 + kCheckBox * b, z, br);
            tma_load_3d_a(sl + kCheckBox * kRowH, mL, base - 4, k0 - 1 + kCheckBox * b, z, br);
        };
        auto trow = [&](int j) {
            return R.base + (uint32_t)((j >> 2) % kCheckSlots) * kCheckSlotA + (uint32_t)(j & 3) * kRowH;
        };
        // skip words (4 cells of a lane) of the rows of a box, two boxes ahead
        auto skip_words = [&](int b, uint32_t(&sk)[kCheckBox]) {
#pragma unroll
            for (int r = 0; r < kCheckBox; ++r) {
                const int j = kCheckBox * b + r;
                sk[r] = (h0 < nxp && j >= 1 && j <= kk)
                            ? __ldg(reinterpret_cast<const uint32_t *>(P.skip + (size_t)(k0 - 1 + j) * nxp + h0))
                            : 0x01010101u;
            }
        };
        uint32_t sk0[kCheckBox], sk1[kCheckBox], sk2[kCheckBox];
        skip_words(0, sk0);
        skip_words(1, sk1);
        issue(0), issue(1), issue(2);
        __syncwarp();
        R.wait(0);
        for (int b = 0; b < nb; ++b) {
            skip_words(b + 2, sk2);
#pragma unroll
            for (int r = 0; r < kCheckBox; ++r) {
                const int j = kCheckBox * b + r;
                if (j < 1 || j > kk) continue;  // warp-uniform
                if (r == kCheckBox - 1) R.wait(b + 1);  // holds row j+1
                const uint32_t rc = trow(j), ru = trow(j - 1), rd = trow(j + 1);
                const uint32_t lo = kCheckBox * kRowH;  // lambda box follows the T box
                const Row4 tc = box_row4(rc, l), lc = box_row4(rc + lo, l);
                const float4 tu = lds4(ru + 16u + 16u * l), td = lds4(rd + 16u + 16u * l);
                const float4 lu = lds4(ru + lo + 16u + 16u * l), ld = lds4(rd + lo + 16u + 16u * l);
                const float tuv[4] = {tu.x, tu.y, tu.z, tu.w}, tdv[4] = {td.x, td.y, td.z, td.w};
                const float luv[4] = {lu.x, lu.y, lu.z, lu.w}, ldv[4] = {ld.x, ld.y, ld.z, ld.w};
                const uint32_t sk = sk0[r];
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const float te = i == 3 ? tc.e : tc.v[i + 1], tw = i == 0 ? tc.w : tc.v[i - 1];
                    const float le = i == 3 ? lc.e : lc.v[i + 1], lw = i == 0 ? lc.w : lc.v[i - 1];
                    const float own = lc.v[i];
                    const float rr = (MODE == kModeReference)
                                         ? leung_qian_ref(tc.v[i], te, tw, tdv[i], tuv[i], le, lw, ldv[i], luv[i], own,
                                                          div, P.eps_adj)
                                         : leung_qian_fast(tc.v[i], te, tw, tdv[i], tuv[i], le, lw, ldv[i], luv[i],
                                                           own, eps_h2);
                    change |= (((sk >> (8 * i)) & 0xffu) == 0) && (rr != own);
                }
            }
#pragma unroll
            for (int r = 0; r < kCheckBox; ++r) sk0[r] = sk1[r], sk1[r] = sk2[r];
            fence_proxy_async_smem();
            __syncwarp();
            if (b >= 1) issue(b + 2);
        }
        change = __any_sync(0xffffffffu, change);
        if (change && l == 0) *(volatile int *)found = 1;
    }
    if (l == 0) ws->cphase = R.phase;
    fence_proxy_async_smem();  // before the next sweep's copies into the ring
    return (__syncthreads_or(change) ? 0 : 1) | (R.err << 1);
}

// whole padded rows, a warp per row, 16-byte accesses (rows are 128-byte aligned)
RZ_DEV void copy_field(const ShotParams &P, const float *src, float *dst) {
    // the padded rows are one contiguous block of ny*nxp floats (nxp a
    // multiple of 4); four 16-byte loads in flight per thread
    const int n4 = P.ny * (P.nxp >> 2), st = blockDim.x;
    const float4 *a = reinterpret_cast<const float4 *>(src);
    float4 *b = reinterpret_cast<float4 *>(dst);
    int i = threadIdx.x;
    for (; i + 3 * st < n4; i += 4 * st) {
        const float4 v0 = __ldcg(a + i), v1 = __ldcg(a + i + st), v2 = __ldcg(a + i + 2 * st),
                     v3 = __ldcg(a + i + 3 * st);
        __stcg(b + i, v0);
        __stcg(b + i + st, v1);
        __stcg(b + i + 2 * st, v2);
        __stcg(b + i + 3 * st, v3);
    }
    for (; i < n4; i += st) __stcg(b + i, __ldcg(a + i));
}

// the adjoint's initial field (init_travel_adj.c:44-57): 0 on the frame,
// 10*TIME inside, the residuals at receiver cells (the receiver cells are
// distinct, each with its last receiver)
RZ_DEV void fill_field(const ShotParams &P, float *F, float v, bool frame0);
RZ_DEV void fill_adjoint_start(const ShotParams &P, float *L, int z) {
    fill_field(P, L, (float)(10.0 * (double)P.time), true);
    __syncthreads();
    for (int i = threadIdx.x; i < P.nrcell; i += blockDim.x)
        L[(size_t)P.rcell_k[i] * P.nxp + P.rcell_h[i]] = P.Tres[(size_t)z * P.ntr + P.rcell_rec[i]];
}

// F := v on every padded row; with frame0 the frame (rows 0 and ny-1,
// columns 0 and nx-1) is 0 instead
RZ_DEV void fill_field(const ShotParams &P, float *F, float v, bool frame0) {
    const int W = blockDim.x >> 5, g = threadIdx.x >> 5, l = threadIdx.x & 31, nq = P.nxp >> 2;
    const int nx = P.nx, ny = P.ny;
    for (int k = g; k < ny; k += W) {
        float4 *row = reinterpret_cast<float4 *>(F + (size_t)k * P.nxp);
        const bool zero_row = frame0 && (k == 0 || k == ny - 1);
        for (int q = l; q < nq; q += 32) {
            float x[4] = {v, v, v, v};
            const int h = 4 * q;
#pragma unroll
            for (int i = 0; i < 4; ++i)
                if (zero_row || (frame0 && (h + i == 0 || h + i == nx - 1))) x[i] = 0.0f;
            row[q] = make_float4(x[0], x[1], x[2], x[3]);
        }
    }
}

// Skewed copies of the converged traveltimes for the adjoint sweeps, plus the
// rows bordering each strip (TMA tiles in, coalesced skew lines out).  The
// work items are (strip s, block G), G = 0..nxb, numbered s*(nxb+1)+G; a warp
// takes items [i0, i1) in order, so the warps of the CTA share the strips.
// The field of shot z under mld goes to the families A / B at dA / dB (the
// shot's TA / TB by default) and its border rows to dEU / dED (none if null).
struct SkewDst {
    float *a, *b, *eu, *ed;
};
RZ_DEV SkewDst skew_dst_t(const ShotParams &P, int z) {
    return {P.TA + (size_t)z * P.sstride, P.TB + (size_t)z * P.sstride, P.EU + (size_t)z * P.estride,
            P.ED + (size_t)z * P.estride};
}
__device__ __noinline__ void relayout_items(const ShotParams &P, Warp &w, const CUtensorMap *mld, int i0, int i1,
                                            SkewDst dst) {
    const int l = w.l, z = w.z;
    float *ring = &w.ws->ring[0][0];
    const int nxb = P.nxb, per = nxb + 1, er = edge_row(P.nxp);
    // tile index G (column block, may be -1 or nxb: zero-filled) -> ring slot
    auto slot_of = [&](int G) { return mod3(G + 1); };
    int s = -1;
    float *ta = nullptr, *tb = nullptr, *ed = nullptr, *eu_next = nullptr;
    auto issue = [&](int G) {  // lane 0
        const int sl = slot_of(G);
        mbar_arrive_expect_tx(&w.mbar[sl], kSlotFloats * 4);
        tma_load_3d(ring + sl * kSlotFloats, mld, kBlk * G, kStrip * s, z, &w.mbar[sl]);
    };
    for (int it = i0; it < i1; ++it) {
        const int G = it % per;
        if (it / per != s) {  // first item of a strip in this range: tiles G-1 and G
            s = it / per;
            ta = dst.a + ((size_t)s * P.qn + kSkewFront) * 32;
            tb = dst.b + ((size_t)s * P.qn + kSkewFront) * 32;
            ed = dst.ed ? dst.ed + (size_t)s * er + kEdgePad : nullptr;
            eu_next = (dst.eu && s + 1 < P.nstrips) ? dst.eu + (size_t)(s + 1) * er + kEdgePad : nullptr;
            fence_proxy_async_smem();  // the slots' earlier generic reads precede the copies
            __syncwarp();
            if (l == 0) {
                issue(G - 1);
                issue(G);
            }
            __syncwarp();
            ring_wait(w, slot_of(G - 1));
        }
        ring_wait(w, slot_of(G));
        // the next block of this strip goes where block G-2 was (read an item ago)
        fence_proxy_async_smem();
        __syncwarp();
        if (l == 0 && G + 1 <= nxb && it + 1 < i1) issue(G + 1);
        const float *t_prev = ring + slot_of(G - 1) * kSlotFloats;
        const float *t_cur = ring + slot_of(G) * kSlotFloats;
        // skew lines q in [32G, 32G+32): family A column q-j, family B column q+j-31
#pragma unroll 8
        for (int qq = 0; qq < 32; ++qq) {
            const int q = kBlk * G + qq;
            const int ca = qq - l;  // column offset relative to tile G (lane = j)
            const int cb = qq + l - 31;
            const float va = ca >= 0 ? t_cur[l * kBlk + ca] : t_prev[l * kBlk + ca + 32];
            const float vb = cb >= 0 ? t_cur[l * kBlk + cb] : t_prev[l * kBlk + cb + 32];
            ta[(size_t)q * 32 + l] = va;
            tb[(size_t)q * 32 + l] = vb;
        }
        if (G < nxb && ed) {
            ed[kBlk * G + l] = t_cur[32 * kBlk + l];                   // row 32s+32 (zero beyond the grid)
            if (eu_next) eu_next[kBlk * G + l] = t_cur[31 * kBlk + l];  // row 32(s+1)-1
        }
        __syncwarp();
    }
}

// The weights of the exact adjoint (or the refinement's residuals) of the
// cells of items [i0, i1) -- (strip s, block G), numbered s*(nxb+1)+G as in
// relayout_items -- computed from the traveltime tiles in the warp's ring:
// blocks G-1, G and G+1 of the strip's 33 rows (the next strip's first row
// included) are in three slots while the item's lines q in [32G, 32G+32) of
// both skew families are written.  Lane l walks its row: at step qq it takes
// column 32G+qq-l (family A) or 32G+qq+l-31 (family B), reads the tile one
// column ahead (anti-diagonal addresses, one bank per lane), gets the rows
// above and below by shuffles (lane 0's upper row from T, lane 31's lower one
// from the tile's 33rd row) and writes its cell of line q: the packed weights
// to TA/TB and (tangent) the residual to RA/RB.  Slowness lines are read
// a few steps ahead; the low parts of refined traveltimes come from their
// skewed copy in RA/RB (lo != null), which this pass only reads.
__device__ __noinline__ void tile_prepare(const ShotParams &P, Warp &w, const CUtensorMap *mld, int z, const float *T,
                                          const float *lo, bool tangent, int i0, int i1) {
    const int l = w.l;
    const uint32_t ring_s = smem_u32(&w.ws->ring[0][0]);
    const int nxb = P.nxb, per = nxb + 1, nx = P.nx, ny = P.ny, nxp = P.nxp, qn = P.qn;
    const int hs = P.src_h[z], ks = P.src_k[z];
    const float big = 3.0e38f;
    float *const pa = P.TA + (size_t)z * P.sstride, *const pb = P.TB + (size_t)z * P.sstride;
    float *const ra = P.RA + (size_t)z * P.sstride, *const rb = P.RB + (size_t)z * P.sstride;
    auto slot_of = [&](int G) { return mod3(G + 1); };
    int s = -1;
    auto issue = [&](int G) {  // lane 0
        const int sl = slot_of(G);
        mbar_arrive_expect_tx(&w.mbar[sl], kSlotFloats * 4);
        tma_load_3d(&w.ws->ring[0][0] + sl * kSlotFloats, mld, kBlk * G, kStrip * s, z, &w.mbar[sl]);
    };
    // traveltime of tile row r (grid row 32s+r, r = 0..32) at column c, 32G-33 <= c <= 32G+32
    auto tile = [&](int r, int c) -> float {
        const int blk = (c + 64) / kBlk - 2;  // floor(c / 32)
        return lds(ring_s + (uint32_t)slot_of(blk) * kSlotBytes + (uint32_t)(r * kBlk + (c & (kBlk - 1))) * 4u);
    };
    for (int it = i0; it < i1; ++it) {
        const int G = it % per;
        if (it / per != s) {  // first item of a strip in this range: blocks G-1 and G
            s = it / per;
            fence_proxy_async_smem();  // the slots' earlier generic accesses precede the copies
            __syncwarp();
            if (l == 0) {
                issue(G - 1);
                issue(G);
            }
            __syncwarp();
            ring_wait(w, slot_of(G - 1));
            ring_wait(w, slot_of(G));
        }
        // block G+1 (east neighbours of the item's last column, and the next
        // item's block) goes where block G-2 was, read by no step of this item
        const bool nxt = G + 1 <= nxb;
        fence_proxy_async_smem();
        __syncwarp();
        if (l == 0 && nxt) issue(G + 1);
        __syncwarp();
        bool waited = !nxt;
        const int row = kStrip * s + l;
        const size_t line0 = ((size_t)s * qn + kSkewFront + (size_t)kBlk * G) * 32 + l;  // line q = 32G, lane l
        auto family = [&](auto fam_tag) {
            constexpr bool FA = decltype(fam_tag)::value;
            float *pw = (FA ? pa : pb) + line0;
            float *pr = (FA ? ra : rb) + line0;
            const float *sl = (FA ? P.SA : P.SB) + line0;
            auto col = [&](int qq) { return FA ? kBlk * G + qq - l : kBlk * G + qq + l - (kStrip - 1); };
            // lanes 0 / 31: the traveltime (lane 0) and low part of the row
            // above / below the strip at the cell's column (lane 31's
            // traveltime comes from the tile's 33rd row)
            auto edge_t = [&](int c) -> float {
                return (l == 0 && row < ny && row > 0 && c >= 0 && c < nx) ? __ldcg(T + (size_t)(row - 1) * nxp + c)
                                                                         : big;
            };
            auto edge_lo = [&](int c) -> float {
                if (!lo || row >= ny || c < 0 || c >= nx) return 0.f;
                if (l == 0) return row > 0 ? __ldcg(lo + (size_t)(row - 1) * nxp + c) : 0.f;
                if (l == kStrip - 1) return row < ny - 1 ? __ldcg(lo + (size_t)(row + 1) * nxp + c) : 0.f;
                return 0.f;
            };
            float prev = tile(l, col(0) - 1), cur = tile(l, col(0));
            float lprev = lo ? __ldcg(pr - 32) : 0.f;  // low parts of lines q-1 ..
            float sv[kPrepAhead], lv[kPrepAhead], et[kPrepAhead], el[kPrepAhead];
#pragma unroll
            for (int i = 0; i < kPrepAhead; ++i) {
                sv[i] = __ldg(sl + 32 * i);
                lv[i] = lo ? __ldcg(pr + 32 * i) : 0.f;
                et[i] = edge_t(col(i));
                el[i] = edge_lo(col(i));
            }
            for (int q8 = 0; q8 < kBlk; q8 += kPrepAhead) {
                // the next group's lines (past the item: its neighbours' lines, inside the stream)
                float sn[kPrepAhead], ln8[kPrepAhead], etn[kPrepAhead], eln[kPrepAhead];
#pragma unroll
                for (int i = 0; i < kPrepAhead; ++i) {
                    sn[i] = __ldg(sl + 32 * (q8 + kPrepAhead + i));
                    ln8[i] = lo ? __ldcg(pr + 32 * (q8 + kPrepAhead + i)) : 0.f;
                    etn[i] = edge_t(col(q8 + kPrepAhead + i));
                    eln[i] = edge_lo(col(q8 + kPrepAhead + i));
                }
#pragma unroll
                for (int i = 0; i < kPrepAhead; ++i) {
                    const int qq = q8 + i;
                    if (qq == kBlk - 1 && !waited) {  // the last step reads column 32G+32
                        ring_wait(w, slot_of(G + 1));
                        waited = true;
                    }
                    const int c = col(qq);
                    const float next = tile(l, c + 1);
                    const float lcur = lv[i], lnext = i < kPrepAhead - 1 ? lv[i + 1] : ln8[0];
                    const bool valid = row < ny && c >= 0 && c < nx;
                    // rows above / below: family A lines q-1 / q+1 of lanes l-1 / l+1,
                    // family B lines q+1 / q-1
                    float tn = __shfl_up_sync(0xffffffffu, FA ? prev : next, 1);
                    float ts = __shfl_down_sync(0xffffffffu, FA ? next : prev, 1);
                    float lnn = __shfl_up_sync(0xffffffffu, FA ? lprev : lnext, 1);
                    float lss = __shfl_down_sync(0xffffffffu, FA ? lnext : lprev, 1);
                    const float t32 = tile(kStrip, c);  // row 32s+32 (lane 31's lower row)
                    if (l == 0) tn = et[i], lnn = el[i];
                    if (l == kStrip - 1) ts = row < ny - 1 ? t32 : big, lss = el[i];
                    if (row == ny - 1) ts = big, lss = 0.f;
                    CellNb nb;
                    nb.tc = cur;
                    nb.tw = c > 0 ? prev : big;
                    nb.te = c < nx - 1 ? next : big;
                    nb.tn = tn, nb.ts = ts;
                    nb.lw = c > 0 ? lprev : 0.f;
                    nb.le = c < nx - 1 ? lnext : 0.f;
                    nb.ln = lnn, nb.ls = lss;
                    ExactCoef cf{0.f, 0.f, 0.f};
                    float r = 0.f;
                    if (valid) {
                        const bool src = c == hs && row == ks;
                        cf = exact_coef_nb(nb, sv[i], P.dh, src);
                        if (tangent) r = cell_residual_nb(nb, sv[i], P.dh, src);
                    }
                    pw[(size_t)qq * 32] = pack_weights(cf);
                    if (tangent) pr[(size_t)qq * 32] = r;
                    prev = cur, cur = next, lprev = lcur;
                }
#pragma unroll
                for (int i = 0; i < kPrepAhead; ++i) sv[i] = sn[i], lv[i] = ln8[i], et[i] = etn[i], el[i] = eln[i];
            }
        };
        family(BoolTag<true>{});
        family(BoolTag<false>{});
    }
}

// Exact discrete adjoint preparation (not in the reference): signed weights
// of every cell on its upwind neighbours (exact_coef) in the skewed layout of
// the sweeps (both weights of a cell packed in one float in TA/TB, the z
// weights of the rows bordering each strip in EU/ED), dJ/dT at the receiver
// cells (RA/RB, the residuals of each cell's receivers summed in receiver
// order), mu = 0.  tangent: the traveltime refinement's system instead -- the
// residual r of every cell (cell_residual_nb) in RA/RB.  The cells' weights
// come from the traveltime tiles (tile_prepare); the border rows' z weights
// and the receiver terms are gathered from the row-major fields.
__device__ __noinline__ void exact_prepare(const ShotParams &P, Warp &w, const CUtensorMap *mld,
                                           const CUtensorMap *mlo, int z, const float *T, float *L, bool tangent) {
    const int tid = threadIdx.x, nthr = blockDim.x;
    const int g = tid >> 5, W = nthr >> 5;
    const int hs = P.src_h[z], ks = P.src_k[z];
    const int nx = P.nx, ny = P.ny, nxp = P.nxp, qn = P.qn;
    float *ra = P.RA + (size_t)z * P.sstride, *rb = P.RB + (size_t)z * P.sstride;
    // low parts of refined traveltimes (the exact adjoint after a refinement):
    // skewed into RA/RB for the weights, then overwritten by the receiver terms
    const float *lo = (P.refine && !tangent) ? P.Told + (size_t)z * P.fstride : nullptr;
    const int er = edge_row(nxp);
    {
        const int items = P.nstrips * (P.nxb + 1);
        const int per_warp = (items + W - 1) / W;
        const int i0 = min(items, g * per_warp), i1 = min(items, (g + 1) * per_warp);
        if (lo) {
            relayout_items(P, w, mlo, i0, i1, SkewDst{ra, rb, nullptr, nullptr});
            __syncthreads();
        }
        tile_prepare(P, w, mld, z, T, lo, tangent, i0, i1);
    }
    __syncthreads();
    // lines no item covers: no dependence (packed 2.0), no residual; the exact
    // adjoint's receiver terms start from zero everywhere
    {
        const int lead = kSkewFront, tail0 = kSkewFront + kBlk * (P.nxb + 1), nout = lead + (qn - tail0);
        for (int i = tid; i < 2 * P.nstrips * nout * 32; i += nthr) {
            const int lane = i & 31, u = i >> 5, fam = u / (P.nstrips * nout), v = u - fam * (P.nstrips * nout);
            const int st = v / nout, k = v - st * nout, q = k < lead ? k : tail0 + (k - lead);
            const size_t o = ((size_t)st * qn + q) * 32 + lane;
            (fam ? P.TB : P.TA)[(size_t)z * P.sstride + o] = 2.0f;
            if (tangent) (fam ? rb : ra)[o] = 0.f;
        }
        if (!tangent) {
            float4 *a4 = reinterpret_cast<float4 *>(ra), *b4 = reinterpret_cast<float4 *>(rb);
            for (size_t i = tid; i < P.sstride / 4; i += nthr) a4[i] = b4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
    __syncthreads();
    // z weights of the rows above (EU) and below (ED) each strip (the exact
    // adjoint's sweeps read them; the refinement's use only a cell's own weights)
    for (int i = tid; i < (tangent ? 0 : P.nstrips * nxp); i += nthr) {
        const int s = i / nxp, col = i - s * nxp;
        const int ru = kStrip * s - 1, rd = kStrip * s + kStrip;
        float vu = 0.f, vd = 0.f;
        if (col < nx) {
            // slowness of these cells from the skewed copy (family A, q = h + j)
            if (ru >= 0) {
                const size_t o = ((size_t)(s - 1) * qn + (col + 31) + kSkewFront) * 32 + 31;
                vu = exact_coef(T, nxp, nx, ny, col, ru, __ldg(P.SA + o), P.dh, col == hs && ru == ks, lo).wz;
            }
            if (rd < ny) {
                const size_t o = ((size_t)(s + 1) * qn + col + kSkewFront) * 32;
                vd = exact_coef(T, nxp, nx, ny, col, rd, __ldg(P.SA + o), P.dh, col == hs && rd == ks, lo).wz;
            }
        }
        P.EU[(size_t)z * P.estride + (size_t)s * er + kEdgePad + col] = vu;
        P.ED[(size_t)z * P.estride + (size_t)s * er + kEdgePad + col] = vd;
    }
    fill_field(P, L, 0.0f, false);
    __syncthreads();
    if (tangent) return;
    for (int i = tid; i < P.nxcell; i += nthr) {
        const int h = P.xcell_h[i], k = P.xcell_k[i];
        float sum = 0.f;
        for (int r = P.xcell_off[i]; r < P.xcell_off[i + 1]; ++r) sum += P.Tres[(size_t)z * P.ntr + P.xcell_rec[r]];
        const int s = k >> 5, j = k & 31;
        ra[((size_t)s * qn + (h + j) + kSkewFront) * 32 + j] = sum;
        rb[((size_t)s * qn + (h - j + 31) + kSkewFront) * 32 + j] = sum;
    }
}

// refined traveltimes: T := RN(T + delta), Told := (T - RN(T + delta)) + delta
// (exact: |delta| <= |T| away from the source, where both are 0)
RZ_DEV void split_refined(const ShotParams &P, float *T, const float *D, float *Tlo) {
    const int W = blockDim.x >> 5, g = threadIdx.x >> 5, l = threadIdx.x & 31, nq = P.nxp >> 2;
    for (int k = g; k < P.ny; k += W) {
        float4 *t = reinterpret_cast<float4 *>(T + (size_t)k * P.nxp);
        const float4 *d = reinterpret_cast<const float4 *>(D + (size_t)k * P.nxp);
        float4 *lo = reinterpret_cast<float4 *>(Tlo + (size_t)k * P.nxp);
        for (int q = l; q < nq; q += 32) {
            const float4 a = __ldcg(t + q), b = __ldcg(d + q);
            float4 hi, rem;
            hi.x = __fadd_rn(a.x, b.x), rem.x = __fadd_rn(__fsub_rn(a.x, hi.x), b.x);
            hi.y = __fadd_rn(a.y, b.y), rem.y = __fadd_rn(__fsub_rn(a.y, hi.y), b.y);
            hi.z = __fadd_rn(a.z, b.z), rem.z = __fadd_rn(__fsub_rn(a.z, hi.z), b.z);
            hi.w = __fadd_rn(a.w, b.w), rem.w = __fadd_rn(__fsub_rn(a.w, hi.w), b.w);
            t[q] = hi;
            lo[q] = rem;
        }
    }
}

// ---------------------------------------------------------------------------
// the shot kernel
// ---------------------------------------------------------------------------
// Shared-memory layout of a CTA of Wb warps, and its (re)initialisation: ring
// and hand-off barriers armed at phase 0, control words and completed-sweep
// counters cleared.  reinit invalidates the barriers of the previous job.
RZ_DEV CtaShared carve_smem(unsigned char *smem_raw, int Wb) {
    CtaShared sh;
    size_t o = 0;
    sh.w = reinterpret_cast<WarpShared *>(smem_raw);
    o = sizeof(WarpShared) * Wb;
    o = align_up(o, 8);
    sh.mbar = reinterpret_cast<uint64_t *>(smem_raw + o);
    o += sizeof(uint64_t) * kRing * Wb;
    o = align_up(o, 8);
    sh.red = reinterpret_cast<double *>(smem_raw + o);
    o += sizeof(double) * Wb;
    sh.ctl = reinterpret_cast<int *>(smem_raw + o);
    sh.done = sh.ctl + 8;
    return sh;
}

RZ_DEV void init_cta(const CtaShared &sh, int Wb, bool reinit) {
    const int tid = threadIdx.x, g = tid >> 5, l = tid & 31;
    if (l == 0) {
        for (int i = 0; i < kRing; ++i) {
            if (reinit) mbar_inval(&sh.mbar[g * kRing + i]);
            mbar_init(&sh.mbar[g * kRing + i], 1);
        }
    }
    handoff_init(&sh.w[g], reinit);
    if (l == 0) {
        for (int i = 0; i < kCheckSlots; ++i) {
            if (reinit) mbar_inval(&sh.w[g].cbar[i]);
            mbar_init(&sh.w[g].cbar[i], 1);
        }
        sh.w[g].cphase = 0;
    }
    if (tid < 7) sh.ctl[tid] = 0;  // ctl[7] carries the job number of a persistent CTA
    if (tid < Wb) sh.done[tid] = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    __syncthreads();
}

// The linear sweeps stage their second stream (RQS) when the CTA has enough
// warps that do not sweep (each lends 12 one-KB slots of its 12.4 KB ring);
// each choice is its own instantiation, so neither carries the other's
// registers.
template <int DX, int DY, bool ADJ, int MODE, int DIV>
__device__ __forceinline__ void sweep_dispatch(const ShotParams &P, Warp &w, const CUtensorMap *mld,
                                               const CUtensorMap *mst, float &acc, uint32_t &moved, int band, int W,
                                               const SweepSeq &seq) {
    if constexpr (ADJ && (MODE == kModeExact || MODE == kModeTangent)) {
        if (((int)(blockDim.x >> 5) - W) * 12 >= W) {
            sweep<DX, DY, ADJ, MODE, DIV, true>(P, w, mld, mst, acc, moved, band, W, seq);
            return;
        }
    }
    sweep<DX, DY, ADJ, MODE, DIV, false>(P, w, mld, mst, acc, moved, band, W, seq);
}

// One shot (forward, residuals, adjoint) by a CTA whose warps 0..Wg-1 take
// the strips (further warps of the CTA only join its barriers and the
// cell-parallel loops).
template <int MODE>
__device__ __forceinline__ void run_shot(const ShotParams &P, const ShotMaps &M, int z, const CtaShared &sh, int Wg) {
    const int W = Wg;
    const int tid = threadIdx.x, g = tid >> 5, l = tid & 31;
    const CUtensorMap *pTld = &M.tld;
    if (tid == 0) {
        tma_prefetch_desc(pTld), tma_prefetch_desc(&M.tst), tma_prefetch_desc(&M.lld), tma_prefetch_desc(&M.lst);
        tma_prefetch_desc(&M.tchk), tma_prefetch_desc(&M.lchk), tma_prefetch_desc(&M.schk);
    }

    Warp w;
    w.g = g;
    w.l = l;
    w.z = z;
    w.phase = 0;
    w.err = 0;
    w.ws = &sh.w[g];
    w.ws_down = (g + 1 < W) ? &sh.w[g + 1] : nullptr;
    w.ws_all = sh.w;
    w.done = sh.done;
    w.mbar = &sh.mbar[g * kRing];
    w.abort_word = &sh.ctl[1];

    stamp(P, z, 0);
    if (P.model_bad && *(volatile const int *)P.model_bad != kModelOk) {
        if (tid == 0) {
            P.passes_fwd[z] = 0;
            atomicOr(&P.status[z], ERR_BAD_MODEL);
        }
        return;
    }
    float *T = P.T + (size_t)z * P.fstride;
    float *Told = P.Told + (size_t)z * P.fstride;
    float *L = P.L + (size_t)z * P.fstride;
    const int n = P.nx * P.ny;
    const int nbands = (P.nstrips + W - 1) / W;
    int cta_err = 0;
    SweepSeq seq{nbands == 1 ? 1 : 0, 0, 0, 0};
    // one directional sweep of every band; banded sweeps synchronise the CTA
    // after each band, pipelined ones only at the end of a pass
#define RZ_SWEEP_D(DX_, DY_, ADJ_, MODE_, DIV_, LD_, ST_)                           \
    do {                                                                           \
        for (int b = 0; b < nbands; ++b) {                                         \
            sweep_dispatch<DX_, DY_, ADJ_, MODE_, DIV_>(P, w, LD_, ST_, acc, moved, b, W, seq); \
            if (!seq.pipelined) sweep_barrier(sh);                                 \
        }                                                                          \
        seq.advance(DY_);                                                          \
    } while (0)
#define RZ_SWEEP(DX_, DY_, ADJ_, MODE_, LD_, ST_) RZ_SWEEP_D(DX_, DY_, ADJ_, MODE_, 1, LD_, ST_)

    if (!P.start_adjoint) {
        // ---------------- forward ----------------
        const int hs = P.src_h[z], ks = P.src_k[z];
        const float tinit = (float)(2.0 * (double)P.time);  // zero_travel.c:22
        fill_field(P, T, tinit, false);
        __syncthreads();
        if (tid == 0) T[(size_t)ks * P.nxp + hs] = 0.0f;  // eikonal.c:35-36
        fence_proxy_async_global();
        __syncthreads();

        int pass = 0, swept = 0;
        bool go = true;
        while (go) {
            if (pass >= P.max_passes) {
                cta_err |= ERR_NOCONV_FWD;
                break;
            }
            if (MODE == kModeReference && pass > 0) {  // pass 0 starts from the initial field
                copy_field(P, T, Told);
                fence_proxy_async_global();
                __syncthreads();
            }
            float acc = 0.f;
            uint32_t moved = 0;
            RZ_SWEEP(+1, +1, false, MODE, pTld, &M.tst);
            if (pass == 0) stamp(P, z, 5);
            RZ_SWEEP(-1, +1, false, MODE, pTld, &M.tst);
            RZ_SWEEP(-1, -1, false, MODE, pTld, &M.tst);
            RZ_SWEEP(+1, -1, false, MODE, pTld, &M.tst);
            if (seq.pipelined) __syncthreads();
            ++pass;
            swept += 4;  // directional sweeps
            if (*w.abort_word) break;
            if (MODE == kModeReference) {
                go = ref_continue(P, T, Told, sh, acc, 4.0 * nbands * (P.nx + 1), pass > 1, [&](float *F0) {
                    fill_field(P, F0, tinit, false);
                    __syncthreads();
                    if (tid == 0) F0[(size_t)ks * P.nxp + hs] = 0.0f;
                });
            } else {
                double tot = block_sum((double)acc, sh);
                go = (tot / (double)n) >= (double)P.ttnorm;
            }
            if (go && pass < P.max_passes) {
                const int fx = forward_is_fixpoint<MODE>(P, &M.tchk, &M.schk, z, &sh.w[g], &sh.ctl[2], w.abort_word);
                w.err |= fx >> 1;
                if (fx & 1) {
                    ++pass;  // the next pass would change nothing
                    go = false;
                }
            }
        }
        if (tid == 0) P.passes_fwd[z] = pass;
        if (tid == 0 && P.swept) P.swept[2 * z] = swept;
        if (P.refine && !*w.abort_word) {
            // Traveltime refinement to the FP64 fixpoint (not in the
            // reference): delta = r + W delta with r the float-float residual
            // of every cell and W the weights of the float field, solved by the
            // linear sweeps in the forward orders until a sweep after the first
            // pass moves no cell's delta by more than 1e-6 of its value; then
            // T := RN(T + delta) and Told := the remainder, so T + Told is the
            // refined field.
            __syncthreads();
            stamp(P, z, 7);
            exact_prepare(P, w, pTld, &M.tlo, z, T, L, true);
            fence_proxy_async_global();
            __syncthreads();
            int tp = 0;
            for (bool more = true; more;) {
                if (tp >= P.max_passes) {
                    cta_err |= ERR_NOCONV_FWD;
                    break;
                }
                float acc = 0.f;
                uint32_t moved = 0;
                // whether the sweep (or pass) just run moved no cell by more
                // than 1e-6 of its value (a CTA-wide vote, with the barrier)
                auto sweep_small = [&]() {
                    const int any = __syncthreads_or((int)moved);
                    moved = 0;
                    return any == 0;
                };
                if (tp == 0) {
                    RZ_SWEEP(+1, +1, true, kModeTangent, &M.lld, &M.lst);
                    RZ_SWEEP(-1, +1, true, kModeTangent, &M.lld, &M.lst);
                    RZ_SWEEP(-1, -1, true, kModeTangent, &M.lld, &M.lst);
                    RZ_SWEEP(+1, -1, true, kModeTangent, &M.lld, &M.lst);
                    more = !sweep_small();
                } else {
                    // later passes one sweep at a time, as the exact adjoint's:
                    // the first sweep that moves no cell by more than 1e-6 of
                    // its value ends the solve
                    RZ_SWEEP(+1, +1, true, kModeTangent, &M.lld, &M.lst);
                    more = !sweep_small();
                    if (more) {
                        RZ_SWEEP(-1, +1, true, kModeTangent, &M.lld, &M.lst);
                        more = !sweep_small();
                    }
                    if (more) {
                        RZ_SWEEP(-1, -1, true, kModeTangent, &M.lld, &M.lst);
                        more = !sweep_small();
                    }
                    if (more) {
                        RZ_SWEEP(+1, -1, true, kModeTangent, &M.lld, &M.lst);
                        more = !sweep_small();
                    }
                }
                ++tp;
                if (*w.abort_word) break;
            }
            __syncthreads();
            split_refined(P, T, L, Told);
            fence_proxy_async_global();
            __syncthreads();
        }
        stamp(P, z, 1);

        // ---------------- receivers: picks, residuals, misfit ----------------
        // calc_FA.c:15-18 and calc_FA_res.c:34-72; a muted pick (Tobs<0) gives a
        // zero residual and no misfit contribution.
        {
            float *sq = &sh.w[0].ring[0][0];  // scratch: W*3*1056 >= 3168 floats
            const int chunk = kRing * kSlotFloats;
            double l2 = 0.0;
            for (int base = 0; base < P.ntr; base += chunk) {
                const int m = min(chunk, P.ntr - base);
                for (int i = tid; i < m; i += blockDim.x) {
                    const int r = base + i;
                    const int h = P.rec_h[r], k = P.rec_k[r];
                    const size_t o = (size_t)k * P.nxp + h;
                    const float tm = __ldcg(T + o);
                    // refined traveltimes: T + Told (the low part), residuals in double
                    const float tl = P.refine ? __ldcg(Told + o) : 0.0f;
                    P.Tmod[(size_t)z * P.ntr + r] = tm;
                    const float tob = P.do_residual ? P.Tobs[(size_t)z * P.ntr + r] : -1.0f;
                    float tr = 0.f, q = 0.f;
                    if (P.cotangent) {
                        tr = tob;  // dJ/dTmod given by the caller
                    } else if (P.exact && tob >= 0.0f) {
                        if (P.refine) {
                            const double res = ((double)tm - (double)tob) + (double)tl;
                            tr = __double2float_rn(res);
                            q = __double2float_rn(res * res);
                        } else {
                            tr = __fsub_rn(tm, tob);  // dJ/dTmod of J = 0.5 sum (Tmod - Tobs)^2
                            q = __fmul_rn(tr, tr);
                        }
                    } else if (tob >= 0.0f) {
                        tr = P.refine ? __double2float_rn(((double)tm - (double)tob) + (double)tl) : __fsub_rn(tm, tob);
                        q = __fmul_rn(tr, tr);
                        float gt;
                        bool have = true;
                        if (k <= P.ny - 2) {
                            gt = __fsub_rn(__ldcg(T + o + P.nxp), tm);
                            if (P.refine) gt = __fadd_rn(gt, __fsub_rn(__ldcg(Told + o + P.nxp), tl));
                        } else if (k == P.ny - 1) {
                            gt = __fsub_rn(tm, __ldcg(T + o - P.nxp));
                            if (P.refine) gt = __fadd_rn(gt, __fsub_rn(tl, __ldcg(Told + o - P.nxp)));
                        } else {
                            have = false;
                        }
                        if (have) {
                            gt = __fdiv_rn(gt, P.dh);
                            tr = (fabsf(gt) > 0.0f) ? __fdiv_rn(tr, gt) : 0.0f;
                        }
                    }
                    if (P.do_residual) P.Tres[(size_t)z * P.ntr + r] = tr;
                    sq[i] = q;
                }
                __syncthreads();
                if (MODE == kModeReference) {
                    if (tid == 0)
                        for (int i = 0; i < m; ++i) l2 = __dadd_rn(l2, (double)sq[i]);
                } else {
                    double part = 0.0;
                    for (int i = tid; i < m; i += blockDim.x) part += (double)sq[i];
                    l2 += block_sum(part, sh);
                }
                __syncthreads();
            }
            if (tid == 0 && P.do_residual) P.l2[z] = l2;
        }
        stamp(P, z, 2);


    }

    if (!P.do_adjoint) {
        __syncthreads();
        if (l == 0) atomicOr(&P.status[z], w.err);
        if (tid == 0) atomicOr(&P.status[z], cta_err);
        return;
    }

    // ---------------- adjoint preparation ----------------
    __syncthreads();
    if (*w.abort_word) {
        if (l == 0) atomicOr(&P.status[z], w.err);
        if (tid == 0) atomicOr(&P.status[z], cta_err);
        return;
    }
    if (P.exact) {
        exact_prepare(P, w, pTld, &M.tlo, z, T, L, false);
    } else {
        {
            const int items = P.nstrips * (P.nxb + 1), Wb = (int)(blockDim.x >> 5);
            const int per_warp = (items + Wb - 1) / Wb;
            relayout_items(P, w, pTld, min(items, g * per_warp), min(items, (g + 1) * per_warp), skew_dst_t(P, z));
        }
        fill_adjoint_start(P, L, z);
    }
    fence_proxy_async_global();
    __syncthreads();
    stamp(P, z, 3);

    // ---------------- adjoint ----------------
    int pass = 0, swept = 0;
    bool go = true;
    while (go) {
        if (pass >= P.max_passes) {
            cta_err |= ERR_NOCONV_ADJ;
            break;
        }
        if (MODE == kModeReference && !P.exact && pass > 0) {  // pass 0 starts from the initial field
            copy_field(P, L, Told);
            fence_proxy_async_global();
            __syncthreads();
        }
        float acc = 0.f;
        uint32_t moved = 0;
        bool sweep_stop = false;  // exact adjoint: a sweep of a later pass moved no cell by > 1e-6 of its value
        int nsweeps = 4;          // sweeps this pass runs
        if (P.exact && pass > 0) {
            // After the first pass, one sweep at a time: a sweep visits every
            // cell, so a sweep that changes no cell proves the fixpoint (its
            // updates all saw the final values), and one that moves no cell
            // by more than 1e-6 of its value bounds every cell's residual as a
            // pass of such sweeps would; the remaining sweeps of the pass are
            // left out.  (A grid-wide sum of the changes would not do: a region
            // the solution has not reached yet moves little in such a sum.)
            auto sweep_small = [&]() {
                const int any = __syncthreads_or((int)moved);
                moved = 0;
                return any == 0;
            };
            nsweeps = 1;
            RZ_SWEEP(+1, +1, true, kModeExact, &M.lld, &M.lst);
            sweep_stop = sweep_small();
            if (!sweep_stop) {
                ++nsweeps;
                RZ_SWEEP(+1, -1, true, kModeExact, &M.lld, &M.lst);
                sweep_stop = sweep_small();
            }
            if (!sweep_stop) {
                ++nsweeps;
                RZ_SWEEP(-1, +1, true, kModeExact, &M.lld, &M.lst);
                sweep_stop = sweep_small();
            }
            if (!sweep_stop) {
                ++nsweeps;
                RZ_SWEEP(-1, -1, true, kModeExact, &M.lld, &M.lst);
                sweep_stop = sweep_small();
            }
        } else if (P.exact) {
            // same four orderings as the Leung-Qian sweeps (eikonal_adj.c:43-46)
            RZ_SWEEP(+1, +1, true, kModeExact, &M.lld, &M.lst);
            if (pass == 0) stamp(P, z, 6);
            RZ_SWEEP(+1, -1, true, kModeExact, &M.lld, &M.lst);
            RZ_SWEEP(-1, +1, true, kModeExact, &M.lld, &M.lst);
            RZ_SWEEP(-1, -1, true, kModeExact, &M.lld, &M.lst);
        } else if (MODE == kModeReference && !P.div_fast) {
            RZ_SWEEP_D(+1, +1, true, MODE, 0, &M.lld, &M.lst);
            if (pass == 0) stamp(P, z, 6);
            RZ_SWEEP_D(+1, -1, true, MODE, 0, &M.lld, &M.lst);
            RZ_SWEEP_D(-1, +1, true, MODE, 0, &M.lld, &M.lst);
            RZ_SWEEP_D(-1, -1, true, MODE, 0, &M.lld, &M.lst);
        } else {
            RZ_SWEEP(+1, +1, true, MODE, &M.lld, &M.lst);
            if (pass == 0) stamp(P, z, 6);
            RZ_SWEEP(+1, -1, true, MODE, &M.lld, &M.lst);
            RZ_SWEEP(-1, +1, true, MODE, &M.lld, &M.lst);
            RZ_SWEEP(-1, -1, true, MODE, &M.lld, &M.lst);
        }
        if (seq.pipelined) __syncthreads();
        ++pass;
        swept += nsweeps;
        if (*w.abort_word) break;
        if (P.exact && pass > 1) {
            go = !sweep_stop;
        } else if (P.exact) {
            // the adjoint system is triangular in arrival order: Gauss-Seidel
            // sweeps reach its solution exactly; stop once a pass moves no
            // cell by more than 1e-6 of its value
            go = __syncthreads_or((int)moved) != 0;
        } else if (MODE == kModeReference) {
            go = ref_continue(P, L, Told, sh, acc, 4.0 * nbands * (P.nx + 1), pass > 1, [&](float *F0) {
                fill_adjoint_start(P, F0, z);
            });
        } else {
            double tot = block_sum((double)acc, sh);
            go = (tot / (double)n) >= (double)P.ttnorm;
        }
        if (go && !P.exact && P.skip && pass < P.max_passes) {
            const int fx = (MODE == kModeReference && !P.div_fast)
                               ? adjoint_is_fixpoint<MODE, 0>(P, &M.tchk, &M.lchk, z, &sh.w[g], &sh.ctl[2], w.abort_word)
                               : adjoint_is_fixpoint<MODE, 1>(P, &M.tchk, &M.lchk, z, &sh.w[g], &sh.ctl[2], w.abort_word);
            w.err |= fx >> 1;
            if (fx & 1) {
                ++pass;  // the next pass would change nothing
                go = false;
            }
        }
    }
    if (tid == 0) P.passes_adj[z] = pass;
#undef RZ_SWEEP
#undef RZ_SWEEP_D
    if (tid == 0 && P.swept) P.swept[2 * z + 1] = swept;
    stamp(P, z, 4);
    __syncthreads();
    if (l == 0) atomicOr(&P.status[z], w.err);
    if (tid == 0) atomicOr(&P.status[z], cta_err);
}

// one CTA per shot
template <int MODE>
__global__ void __launch_bounds__(kMaxWarps * 32, 1)
    shot_kernel(const __grid_constant__ ShotParams P, const __grid_constant__ ShotMaps M, int Wg) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int Wb = blockDim.x >> 5;
    if ((int)blockIdx.x >= P.nshots) return;
    const CtaShared sh = carve_smem(smem_raw, Wb);
    init_cta(sh, Wb, false);
    run_shot<MODE>(P, M, blockIdx.x, sh, Wg);
}

// Persistent CTAs over the shots of several grids: each CTA takes the next
// job (grid, shot) from a counter, in the host's largest-first order, until
// none is left.
template <int MODE>
__global__ void __launch_bounds__(kMaxWarps * 32, 1) multi_shot_kernel(const __grid_constant__ MultiParams M) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int Wb = blockDim.x >> 5;
    const CtaShared sh = carve_smem(smem_raw, Wb);
    bool first = true;
    for (;;) {
        if (threadIdx.x == 0) sh.ctl[7] = atomicAdd(M.counter, 1);
        __syncthreads();
        const int job = sh.ctl[7];
        if (job >= M.njobs) break;
        const int2 jb = M.jobs[job];
        init_cta(sh, Wb, !first);
        first = false;
        const MultiGrid &G = M.grid[jb.x];
        run_shot<MODE>(G.P, G.maps, jb.y, sh, G.W);
        __syncthreads();
    }
}

int shot_kernel_warps(int nstrips) {
    const int nb = (nstrips + kMaxWarps - 1) / kMaxWarps;  // bands per sweep
    return (nstrips + nb - 1) / nb;                         // warps per CTA, bands balanced
}

// Warps of a CTA whose W warps sweep: further warps idle through the sweeps
// but share the cell-parallel phases (fixpoint checks, field fills); the CTA
// grows while as many CTAs fit on an SM as with W warps.
template <class K>
static cudaError_t block_warps(K kern, int W, int *Wb_out) {
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (!e) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (!e && shot_kernel_smem(W) > (size_t)optin) e = cudaErrorInvalidConfiguration;
    if (!e) e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)std::min(shot_kernel_smem(kMaxWarps), (size_t)optin));
    int base = 0;
    if (!e) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&base, kern, 32 * W, shot_kernel_smem(W));
    if (e) return e;
    int Wb = W;
    for (int v = W + 1; v <= kMaxWarps && shot_kernel_smem(v) <= (size_t)optin; ++v) {
        int o = 0;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, kern, 32 * v, shot_kernel_smem(v)))) return e;
        if (o < base) break;
        Wb = v;
    }
    *Wb_out = Wb;
    return cudaSuccess;
}

// block_warps, remembered per kernel and W
// The answer depends on the device (its shared-memory limit): the cache is
// kept per device and shared by host threads under a lock.
constexpr int kMaxCachedDevices = 64;
static std::mutex g_block_warps_mutex;
template <class K>
static cudaError_t block_warps_cached(K kern, int slot, int W, int *Wb) {
    static int cache[kMaxCachedDevices][4][kMaxWarps + 1];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e) return e;
    if (dev < 0 || dev >= kMaxCachedDevices) return block_warps(kern, W, Wb);
    std::lock_guard<std::mutex> lock(g_block_warps_mutex);
    if (cache[dev][slot][W] > 0) {
        *Wb = cache[dev][slot][W];
        return cudaSuccess;
    }
    e = block_warps(kern, W, Wb);
    if (!e) cache[dev][slot][W] = *Wb;
    return e;
}

cudaError_t launch_multi_shot_kernel(const MultiParams &M, int mode, int W, int *nctas, cudaStream_t st) {
    int dev = 0, sms = 0, per_sm = 0, Wb = W;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    auto kern = mode == kModeReference ? multi_shot_kernel<kModeReference> : multi_shot_kernel<kModeFast>;
    if ((e = block_warps_cached(kern, mode == kModeReference ? 2 : 3, W, &Wb))) return e;
    const size_t smem = shot_kernel_smem(Wb);
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * Wb, smem))) return e;
    const int n = std::max(1, std::min(M.njobs, sms * std::max(per_sm, 1)));
    kern<<<n, 32 * Wb, smem, st>>>(M);
    if (nctas) *nctas = n;
    return cudaGetLastError();
}

cudaError_t launch_shot_kernel(const ShotParams &P, int mode, const ShotMaps &M, cudaStream_t st, int warps,
                               int cta_warps) {
    if (P.nstrips < 1) return cudaErrorInvalidValue;
    const int W = warps > 0 ? std::min(std::min(warps, kMaxWarps), P.nstrips) : shot_kernel_warps(P.nstrips);
    int Wb = W;
    cudaError_t e;
    auto kern = mode == kModeReference ? shot_kernel<kModeReference> : shot_kernel<kModeFast>;
    if ((e = block_warps_cached(kern, mode == kModeReference ? 0 : 1, W, &Wb))) return e;
    // a requested CTA width between W and the widest that keeps the occupancy
    if (cta_warps > 0) Wb = std::max(W, std::min(cta_warps, Wb));
    kern<<<P.nshots, 32 * Wb, shot_kernel_smem(Wb), st>>>(P, M, W);
    return cudaGetLastError();
}

}  // namespace rz
