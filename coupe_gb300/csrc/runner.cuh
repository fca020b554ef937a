// The level loop of one Rcb run (host side), templated on dimension, key
// precision and weight type.  It replaces rcb / rcb_recurse
// (coupe/src/algorithms/recursive_bisection.rs:575-705): instead of a
// fork-join over the bisection tree, every tree level is processed at once,
// all of its segments in the same kernel launches.
#pragma once

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "engine.h"
#include "kernels.cuh"

namespace cg {

// NVTX range over a scope (a run, a tree level, an extra pass): the GPU
// counterpart of coupe's tracing spans (recursive_bisection.rs:467-468,
// 590-595).  Visible in Nsight timelines; a no-op without a tool attached.
struct NvtxScope {
    explicit NvtxScope(const char *name) { nvtxRangePushA(name); }
    NvtxScope(const char *what, uint64_t k) {
        char b[48];
        snprintf(b, sizeof(b), "%s %llu", what, (unsigned long long)k);
        nvtxRangePushA(b);
    }
    ~NvtxScope() { nvtxRangePop(); }
    NvtxScope(const NvtxScope &) = delete;
    NvtxScope &operator=(const NvtxScope &) = delete;
};

#define CG_CK(call)                                               \
    do {                                                          \
        cudaError_t e_ = (call);                                  \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call, err);  \
    } while (0)

// Launches a kernel, bracketed by profiler events when profiling is on.
#define CG_LAUNCH(kid, nbytes, ...)                                 \
    do {                                                            \
        C.prof.begin((kid), (nbytes), s);                           \
        __VA_ARGS__;                                                \
        cudaError_t e_ = cudaGetLastError();                        \
        if (e_ != cudaSuccess) return cuda_fail(e_, "launch", err); \
        C.prof.end(s);                                              \
        ++st->kernel_launches;                                      \
    } while (0)

struct Bump {
    char *base;
    size_t off;
    template <class T>
    T *take(size_t count) {
        off = (off + 255) & ~(size_t)255;
        T *p = (T *)(base + off);
        off += count * sizeof(T);
        return p;
    }
};

template <int D, class KT, class WT>
struct Buffers {
    typedef typename KT::T K;
    typedef typename KT::Ord O;
    K *keys[3][3];  // [0]: level-0 keys in input order (kept); [1], [2]: reorder ping-pong
    typename WT::S *w[2];
    uint32_t *idx[2];  // input index of each item (index path only)
    Seg<KT> *segs[2];
    uint32_t *list[2];
    uint64_t *P[2];
    uint32_t *flags;
    uint32_t *hcnt;
    uint64_t *hw;
    O *hinv;
    uint64_t *lb;
    uint64_t *blk;   // per-CTA child counts of the grid form of k_children
    Trav<KT> *trav;  // finished splits of every level (traversal path only)
    uint64_t *lvl;   // [2 (levels + 1)]: segments and items of each level
    RunScalars *rs;
    uint64_t hist_bins;
    // several sets: the set table and the sets of the root segments
    uint64_t *set_off, *set_bmin, *set_bmax, *set_wsum, *set_wabs, *set_minheap;
    uint32_t *set_iters, *set_root, *roots;
    int32_t *set_fs, *set_qb;

    SetTab set_tab(uint32_t count) const {
        SetTab t;
        t.count = count;
        t.off = set_off;
        t.iters = set_iters;
        t.root = set_root;
        t.bmin = set_bmin;
        t.bmax = set_bmax;
        t.wsum = set_wsum;
        t.wabs = set_wabs;
        t.fs = set_fs;
        t.qb = set_qb;
        t.minheap = set_minheap;
        return t;
    }

    size_t carve(Bump &b, uint64_t n, uint64_t scap, uint64_t hb, uint64_t lbcap, bool index_path, bool carry,
                 uint64_t tcap, uint64_t nsets, uint64_t levels) {
        for (int k = 0; k < 3; ++k)
            for (int d = 0; d < 3; ++d) keys[k][d] = d < D ? b.take<K>(n) : nullptr;
        for (int s = 0; s < 2; ++s) {
            w[s] = b.take<typename WT::S>(n);
            idx[s] = carry ? b.take<uint32_t>(n) : nullptr;
            segs[s] = b.take<Seg<KT>>(scap);
            list[s] = b.take<uint32_t>(scap);
            P[s] = b.take<uint64_t>(scap + 1);
        }
        flags = b.take<uint32_t>(scap);
        hcnt = b.take<uint32_t>(hb);
        hw = b.take<uint64_t>(hb * WT::LIMBS);
        hinv = b.take<O>(hb);
        lb = b.take<uint64_t>(lbcap);
        blk = b.take<uint64_t>(2 * (scap / 1024 + 1));
        trav = index_path ? nullptr : b.take<Trav<KT>>(tcap);
        lvl = b.take<uint64_t>(2 * (levels + 1));
        rs = b.take<RunScalars>(1);
        hist_bins = hb;
        set_off = set_bmin = set_bmax = set_wsum = set_wabs = set_minheap = nullptr;
        set_iters = set_root = roots = nullptr;
        set_fs = set_qb = nullptr;
        if (nsets) {
            set_off = b.take<uint64_t>(nsets + 1);
            set_iters = b.take<uint32_t>(nsets);
            set_root = b.take<uint32_t>(nsets);
            roots = b.take<uint32_t>(nsets);
            set_bmin = b.take<uint64_t>(nsets * 3);
            set_bmax = b.take<uint64_t>(nsets * 3);
            set_wsum = b.take<uint64_t>(nsets * 4);
            set_wabs = b.take<uint64_t>(nsets);
            set_fs = b.take<int32_t>(nsets);
            set_qb = b.take<int32_t>(nsets);
            set_minheap = b.take<uint64_t>(nsets);
        }
        return b.off;
    }
};

static inline int occupancy_grid(const void *fn, int sms, int block, size_t smem) {
    int per = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, block, smem) != cudaSuccess || per < 1) per = 1;
    return per * sms;
}

// Segments per k_decide CTA (one warp each): as few as keep the grid within
// the `resident` CTAs of one wave, so that short lists spread their
// decisions, whose FP64 work bounds them, over the SMs (256 segments: 256
// CTAs of one working warp rather than 32 CTAs of eight).
static inline uint32_t decide_segs_per_cta(uint64_t S, int resident) {
    const uint64_t r = (uint64_t)std::max(1, resident);
    return (uint32_t)std::min<uint64_t>(NWARPS, std::max<uint64_t>(1, (S + r - 1) / r));
}

// What the set-up of a run hands to its level loop.
struct RunSetup {
    uint64_t n = 0, iters = 0, lbcap = 0, bytes = 0;
    uint32_t nsets = 1;   // > 1: a batched run (set table in the buffers)
    uint32_t nroots = 1;  // root segments on level 0
    uint64_t v0 = 0;      // items of the root segments
    bool index_path = false;  // part ids from the segments (k_assign), not a traversal
    bool carry = false;       // reorders carry input indices (index path, band form)
    Mat M;                    // the basis change k_convert applied
    cudaStream_t s = nullptr;
    RunScalars *h_rs = nullptr;
    int g_stream = 0;
    std::vector<uint64_t> smax, vmax;  // per level: most segments, and items
};

// The level loop of one run; WT is the caller's weight type (it sizes the
// buffers), WL the type the loop reads (WT, or its 16-bit copy WtC16<WT>).
template <int D, class KT, class WT, class WL>
int run_levels(DevCtx &C, const RunArgs &a, coupe_gpu_stats *st, std::string *err, Buffers<D, KT, WT> &B,
               const RunSetup &R0, const typename WL::S *w_in) {
    typedef typename KT::T K;
    typedef typename WL::S WS;
    const Tuning &tu = tuning();
    const uint64_t n = R0.n, iters = R0.iters;
    const bool index_path = R0.index_path, carry = R0.carry;
    cudaStream_t s = R0.s;
    const BandSrc bs = make_band_src(a.d_points, R0.M, D, &B.rs->band_points);
    RunScalars *h_rs = R0.h_rs;
    const int g_stream = R0.g_stream;
    uint64_t bytes = R0.bytes;
    const int nbk_max = std::min(hist_max_nbk<WL>(), std::max(1, tu.max_nbk));
    const size_t r_smem = reorder_smem<D, KT, WL>(carry);
    if constexpr (KT::BAND) {
        CG_CK(cudaFuncSetAttribute((const void *)k_traverse_band<D>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)TRAV_SMEM_MAX));
    } else {
        CG_CK(cudaFuncSetAttribute((const void *)k_traverse_smem<D, KT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)TRAV_SMEM_MAX));
    }
    const void *reorder_fn = carry ? (const void *)k_reorder<D, KT, WL, true> : (const void *)k_reorder<D, KT, WL, false>;
    CG_CK(cudaFuncSetAttribute(reorder_fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)r_smem));
    const int g_reorder = occupancy_grid(reorder_fn, C.sms, BLOCK, r_smem);
    // levels of small segments (below SMALL_SEG_ITEMS items on average) use
    // the double-buffered k_reorder_small
    const size_t rs_smem = small_reorder_smem<D, KT, WL>(carry);
    const void *reorder_small_fn =
        carry ? (const void *)k_reorder_small<D, KT, WL, true> : (const void *)k_reorder_small<D, KT, WL, false>;
    CG_CK(cudaFuncSetAttribute(reorder_small_fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rs_smem));
    const int g_reorder_small = occupancy_grid(reorder_small_fn, C.sms, BLOCK, rs_smem);
    constexpr uint64_t SMALL_SEG_ITEMS = 4 * R_TILE;
    const uint64_t per_cta = (uint64_t)std::max(1, tu.reorder_chunks_per_cta);
    // reorder chunks over the V items of a level's segments, for a grid of g CTAs
    auto chunk_of = [&](uint64_t V, int g) {
        uint64_t c = std::max<uint64_t>(R_TILE, (V + (uint64_t)g * per_cta - 1) / ((uint64_t)g * per_cta));
        return (c + R_TILE - 1) / R_TILE * R_TILE;
    };
    const bool multi = R0.nsets > 1;
    const SetTab sets = B.set_tab(R0.nsets);
    const int32_t *set_fs = multi && WL::LIMBS > 1 ? B.set_fs : nullptr;
    const int32_t *set_qb = multi && WL::LIMBS > 1 ? B.set_qb : nullptr;
    const int approx = tu.exact_f64_hist ? 0 : 1;
    int g_hist = occupancy_grid((const void *)k_hist<KT, WL>, C.sms, BLOCK, 0);
    if (tu.hist_ctas_per_sm > 0) g_hist = std::min(g_hist, tu.hist_ctas_per_sm * C.sms);
    g_hist *= std::max(1, std::min(tu.hist_waves, 16));
    const int g_decide = occupancy_grid((const void *)k_decide<KT, WL>, C.sms, BLOCK, 0);
    if (multi) {
        CG_LAUNCH(KID_ROOT, 0,
                  k_roots<KT, WL><<<(R0.nroots + 255) / 256, 256, 0, s>>>(B.segs[0], B.list[0], B.P[0], B.roots,
                                                                           R0.nroots, D, sets, B.rs, approx,
                                                                           B.lvl));
    } else {
        CG_LAUNCH(KID_ROOT, 0,
                  k_root<KT, WL><<<1, 1, 0, s>>>(B.segs[0], B.list[0], B.P[0], n, D, B.rs, approx, B.lvl));
    }
    const uint64_t sk = sizeof(K), sw = sizeof(WS), si = carry ? 4 : 0;

    // Per-level bounds known on the host: segments S_max (a level holds at
    // most min(2^L, n_k) segments of each set still splitting) and items V
    // (every item of a set still splitting is in one of its segments).  The
    // level's kernels read the actual counts from the device
    // (Buffers::lvl, written by the root kernel and by each level's
    // children), so the host queues a whole run
    // without waiting: grids, bins and recorded-split offsets are sized by
    // S_max.  A split that needs more passes than the two queued per level
    // halts the queued kernels after it (RunScalars::stall); the host then
    // finishes that level with more passes and continues level by level,
    // waiting for each (the option sync_levels forces that from the start).
    const std::vector<uint64_t> &smax = R0.smax, &vmax = R0.vmax;
    LevelOffsets lv;
    uint64_t trav_used = 0;
    for (uint64_t L = 0; L < iters; ++L) {
        lv.off[L < (uint64_t)MAX_TRAV_LEVELS ? L : 0] = index_path ? 0 : trav_used;
        if (!index_path) trav_used += smax[L];
    }
    // bins per segment: as many bisection steps per pass as the budget allows
    auto pick_nbk = [&](uint64_t nseg) {
        int k = nbk_max;
        while (k > 1 && nseg * (1ull << k) > B.hist_bins) --k;
        return k;
    };
    int err_level = -1;  // level at whose synchronisation a device check was first seen
    Hist<KT, WL> H{B.hcnt, B.hw, B.hinv};
    // buffers of level L: segment tables and weights alternate; keys are the
    // kept level-0 copy on level 0, then the two reorder buffers in turn
    auto key_buf = [](uint64_t L) { return L == 0 ? 0 : (L % 2 == 1 ? 1 : 2); };
    auto seg_buf = [](uint64_t L) { return (int)(L & 1); };

    // Queues level L.  sync: wait for its decisions and run further passes
    // while splits still search; resume: its two queued passes already ran
    // (a halted queued run), so start with the further passes.
    // speculative passes queued after each level's first one (1; one more
    // for the levels queued again after a halt), and per level the list
    // that holds the segments still searching after them
    int nspec = 1;
    std::vector<int> active_list(iters, 0);
    auto level = [&](uint64_t L, bool sync, bool resume) -> int {
        NvtxScope level_range("rcb level", L);
        const int coord = (int)(L % D);
        const uint64_t S_max = smax[L], V = vmax[L];
        const int nbk = pick_nbk(S_max);
        const uint64_t NB = 1ull << nbk;
        const int kb = key_buf(L), sb = seg_buf(L);
        const bool level0 = L == 0;  // level 0 reads the caller's weights and implicit indices
        const K *kc = B.keys[kb][coord];
        const WS *wc = level0 ? w_in : (const WS *)B.w[sb];
        const uint32_t *ic = level0 ? nullptr : B.idx[sb];
        Seg<KT> *segs = B.segs[sb];
        const bool last = L + 1 == iters;
        const int snext = sb ^ 1;
        Trav<KT> *trav_l = index_path ? nullptr : B.trav + lv.off[L];
        const uint64_t *S_dev = &B.lvl[2 * L];
        const uint64_t *V_dev = &B.lvl[2 * L + 1];
        // band form: the items' input indices, for coordinates in the band
        const uint32_t *hsrc = KT::BAND ? ic : nullptr;
        const bool fuse = S_max < CHILD_GRID_MIN;
        auto children = [&]() {
            const int wr = last ? 0 : 1;
            if (fuse) {
                CG_LAUNCH(KID_CHILDREN, 0,
                          k_children<KT, WL><<<1, 1024, 0, s>>>(segs, 0u, coord, D, wr, (uint32_t)L, B.segs[snext],
                                                                B.list[0], B.P[0], trav_l, B.rs, sets, CHILD_ALL,
                                                                B.blk, S_dev, B.lvl));
                return (int)COUPE_ERR_OK;
            }
            const unsigned g = (unsigned)((S_max + 1023) / 1024);
            for (int ph : {(int)CHILD_COUNT, (int)CHILD_SCAN, (int)CHILD_WRITE}) {
                CG_LAUNCH(KID_CHILDREN, 0,
                          k_children<KT, WL><<<ph == CHILD_SCAN ? 1u : g, 1024, 0, s>>>(
                              segs, 0u, coord, D, wr, (uint32_t)L, B.segs[snext], B.list[0], B.P[0], trav_l, B.rs,
                              sets, ph, B.blk, S_dev, B.lvl));
            }
            return (int)COUPE_ERR_OK;
        };
        const uint32_t decide_spc = decide_segs_per_cta(S_max, g_decide);
        const unsigned decide_grid = (unsigned)((S_max + decide_spc - 1) / decide_spc);
        ChildArgs<KT> no_ch;
        std::memset(&no_ch, 0, sizeof(no_ch));
        const uint64_t decide_bytes = S_max * NB * (4 + 8 * WL::LIMBS + sizeof(typename KT::Ord));
        if (!resume) {
            // levels below CHILD_GRID_MIN segments build their children in
            // the last CTA of the speculative decide (when no segment is
            // searching any more)
            ChildArgs<KT> ch = no_ch;
            ch.on = fuse ? 1 : 0;
            ch.stall_level = sync ? 0u : (uint32_t)(L + 1);
            ch.S_ptr = S_dev;
            ch.lvl = B.lvl;
            ch.coord = coord;
            ch.D = D;
            ch.write = last ? 0 : 1;
            ch.level = (uint32_t)L;
            ch.next = B.segs[snext];
            ch.next_list = B.list[0];
            ch.next_P = B.P[0];
            ch.trav = trav_l;
            ch.sets = sets;
            // First pass over every point of the level, its decisions, and
            // the list of segments still searching (list[1]).
            CG_CK(cudaMemsetAsync(B.hcnt, 0, S_max * NB * sizeof(uint32_t), s));
            CG_CK(cudaMemsetAsync(B.hw, 0, S_max * NB * WL::LIMBS * sizeof(uint64_t), s));
            CG_CK(cudaMemsetAsync(B.hinv, 0, S_max * NB * sizeof(typename KT::Ord), s));
            CG_LAUNCH(KID_HIST, V * (sk + sw),
                      k_hist<KT, WL><<<g_hist, BLOCK, 0, s>>>(segs, B.list[0], B.P[0], 0u, kc, wc, H, nbk, n, B.rs,
                                                              S_dev, hsrc, bs, coord, segs, set_fs, set_qb));
            ++st->hist_passes;
            st->hist_points += V;
            bytes += V * (sk + sw);
            CG_LAUNCH(KID_DECIDE, decide_bytes,
                      k_decide<KT, WL><<<decide_grid, BLOCK, 0, s>>>(segs, B.list[0], 0u, H, nbk, a.tolerance,
                                                                     B.flags, B.rs, S_dev, set_fs, set_qb, B.list[1],
                                                                     B.P[1], no_ch, decide_spc));
            // Speculative passes over the list the last scan left: their
            // kernels read its count and return at once when no segment is
            // searching.  The lists alternate; the last pass's decide builds
            // the children (next level's list in list[0], written only when
            // its own scan, into the other list, found nothing searching).
            const int ns = sync ? 1 : nspec;
            int li = 1;
            for (int p = 0; p < ns; ++p) {
                const bool final_pass = p + 1 == ns;
                CG_LAUNCH(KID_HIST, 0,
                          k_hist<KT, WL><<<g_hist, BLOCK, 0, s>>>(segs, B.list[li], B.P[li], 0u, kc, wc, H, nbk, n,
                                                                  B.rs, &B.rs->nactive, hsrc, bs, coord, segs, set_fs,
                                                                  set_qb));
                ++st->hist_passes;
                CG_LAUNCH(KID_DECIDE, decide_bytes,
                          k_decide<KT, WL><<<decide_grid, BLOCK, 0, s>>>(segs, B.list[li], 0u, H, nbk, a.tolerance,
                                                                         B.flags, B.rs, &B.rs->nactive, set_fs, set_qb,
                                                                         B.list[li ^ 1], B.P[li ^ 1],
                                                                         final_pass ? ch : no_ch, decide_spc));
                li ^= 1;
            }
            active_list[L] = li;
            // k_children returns at once if a segment is still searching
            if (!fuse) {
                const int rc_ = children();
                if (rc_ != COUPE_ERR_OK) return rc_;
            }
        }
        if (sync) {
            CG_CK(cudaMemcpyAsync(h_rs, B.rs, sizeof(RunScalars), cudaMemcpyDeviceToHost, s));
            CG_CK(cudaStreamSynchronize(s));
            ++st->host_syncs;
            if (h_rs->err) {
                err_level = (int)L;
                return -1;
            }
            // rare: splits that need more steps than the queued passes replay
            int li = active_list[L], extra = 0;
            bool more = false;
            while (h_rs->nactive > 0) {
                NvtxScope pass_range("rcb extra pass", (uint64_t)extra);
                more = true;
                if (++extra > 4096) {
                    *err = "a split did not finish after 4096 passes";
                    return COUPE_ERR_CRASH;
                }
                const uint64_t nlist = h_rs->nactive;
                CG_LAUNCH(KID_HIST, h_rs->total_active * (sk + sw),
                          k_hist<KT, WL><<<g_hist, BLOCK, 0, s>>>(segs, B.list[li], B.P[li], (uint32_t)nlist, kc, wc,
                                                                  H, nbk, n, B.rs, nullptr, hsrc, bs, coord, segs,
                                                                  set_fs, set_qb));
                ++st->hist_passes;
                const uint32_t spc = decide_segs_per_cta(nlist, g_decide);
                CG_LAUNCH(KID_DECIDE, nlist * NB * (4 + 8 * WL::LIMBS + sizeof(typename KT::Ord)),
                          k_decide<KT, WL><<<(unsigned)((nlist + spc - 1) / spc), BLOCK, 0, s>>>(
                              segs, B.list[li], (uint32_t)nlist, H, nbk, a.tolerance, B.flags, B.rs, nullptr, set_fs,
                              set_qb, B.list[li ^ 1], B.P[li ^ 1], no_ch, spc));
                li ^= 1;
                CG_CK(cudaMemcpyAsync(h_rs, B.rs, sizeof(RunScalars), cudaMemcpyDeviceToHost, s));
                CG_CK(cudaStreamSynchronize(s));
                ++st->host_syncs;
                if (h_rs->err) {
                    err_level = (int)L;
                    return -1;
                }
            }
            if (more || resume) {
                const int rc_ = children();
                if (rc_ != COUPE_ERR_OK) return rc_;
            }
        }
        if (last) {
            // a host call's pinned id buffer takes the traversal's writes
            // directly (coalesced, over the host link) instead of a copy after
            uint64_t *ids = a.d_part;
            if (a.ids_host && !index_path) {
                ids = a.ids_host;
                if (a.ids_on_host) *a.ids_on_host = true;
            }
            if (multi) {
                CG_LAUNCH(KID_ASSIGN, n * (D * sk + 8),
                          k_traverse_sets<D, KT><<<g_stream, BLOCK, 0, s>>>(B.trav, lv, B.keys[0][0], B.keys[0][1],
                                                                            B.keys[0][2], n, ids, sets, bs, B.rs));
                bytes += n * (D * sk + 8);
            } else if (index_path) {
                CG_LAUNCH(KID_ASSIGN, n * (sk + (ic ? 4 : 0) + 8),
                          k_assign<KT><<<g_stream, BLOCK, 0, s>>>(segs, 0u, n, kc, ic, a.d_part, B.rs, bs, coord,
                                                                  S_dev));
                bytes += n * (sk + (ic ? 4 : 0) + 8);
            } else {
                const uint64_t n_last = trav_used - lv.off[iters - 1];
                const size_t tsm = KT::BAND ? trav_band_smem_bytes(trav_used, n_last)
                                            : trav_smem_bytes<KT>(trav_used, n_last);
                if (tsm <= TRAV_SMEM_MAX) {
                    if constexpr (KT::BAND) {
                        // one resident wave: each CTA stages the table once
                        const int g_trav = std::min<int>(
                            g_stream, occupancy_grid((const void *)k_traverse_band<D>, C.sms, BLOCK, tsm));
                        CG_LAUNCH(KID_ASSIGN, n * (D * sk + 8),
                                  k_traverse_band<D><<<g_trav, BLOCK, tsm, s>>>(
                                      B.trav, (uint32_t)trav_used, lv, (int)iters, B.keys[0][0], B.keys[0][1],
                                      B.keys[0][2], n, ids, B.rs, bs));
                    } else {
                        CG_LAUNCH(KID_ASSIGN, n * (D * sk + 8),
                                  k_traverse_smem<D, KT><<<g_stream, BLOCK, tsm, s>>>(
                                      B.trav, (uint32_t)trav_used, lv, (int)iters, B.keys[0][0], B.keys[0][1],
                                      B.keys[0][2], n, ids, B.rs, bs));
                    }
                } else {
                    CG_LAUNCH(KID_ASSIGN, n * (D * sk + 8),
                              k_traverse<D, KT><<<g_stream, BLOCK, 0, s>>>(B.trav, trav_used, lv, (int)iters,
                                                                           B.keys[0][0], B.keys[0][1], B.keys[0][2],
                                                                           n, ids, B.rs, bs));
                }
                bytes += n * (D * sk + 8);
            }
            st->levels = L + 1;
            return COUPE_ERR_OK;
        }
        const bool small_segs = tu.reorder_kernel == 0 ? V < S_max * SMALL_SEG_ITEMS : tu.reorder_kernel == 2;
        const int g_r = small_segs ? g_reorder_small : g_reorder;
        const uint64_t chunk = chunk_of(V, g_r);
        const uint64_t nchunks = (V + chunk - 1) / chunk;
        if (nchunks > R0.lbcap) {
            *err = "internal: more reorder chunks than look-back words";
            return COUPE_ERR_CRASH;
        }
        CG_CK(cudaMemsetAsync(B.lb, 0, nchunks * sizeof(uint64_t), s));
        CG_CK(cudaMemsetAsync(&B.rs->ticket, 0, sizeof(uint64_t), s));
        const int kb_next = key_buf(L + 1);
        ReorderArgs<D, KT, WL> R;
        R.segs = segs;
        R.S = 0;
        R.n = V;
        R.chunk = chunk;
        R.nchunks = nchunks;
        R.coord = coord;
        for (int d = 0; d < 3; ++d) {
            R.ksrc[d] = B.keys[kb][d];
            R.kdst[d] = B.keys[kb_next][d];
        }
        R.wsrc = wc;
        R.wsafe = level0 && w_in == (const WS *)a.d_weights ? 0 : 1;  // the caller's array: element copies
        R.wdst = (WS *)B.w[snext];
        R.isrc = ic;
        R.idst = carry ? B.idx[snext] : nullptr;
        R.bs = bs;
        R.lb = B.lb;
        R.rs = B.rs;
        R.spin_limit = (uint32_t)std::max(0, tu.lookback_spin_limit);
        R.S_ptr = S_dev;
        R.n_ptr = V_dev;
        const uint64_t rbytes = 2 * V * (D * sk + sw + si) - (ic ? 0 : V * si);
        const unsigned r_grid = (unsigned)std::min<uint64_t>(g_r, nchunks);
        if (small_segs) {
            if (carry) {
                CG_LAUNCH(KID_REORDER, rbytes, k_reorder_small<D, KT, WL, true><<<r_grid, BLOCK, rs_smem, s>>>(R));
            } else {
                CG_LAUNCH(KID_REORDER, rbytes, k_reorder_small<D, KT, WL, false><<<r_grid, BLOCK, rs_smem, s>>>(R));
            }
        } else if (carry) {
            CG_LAUNCH(KID_REORDER, rbytes, k_reorder<D, KT, WL, true><<<r_grid, BLOCK, r_smem, s>>>(R));
        } else {
            CG_LAUNCH(KID_REORDER, rbytes, k_reorder<D, KT, WL, false><<<r_grid, BLOCK, r_smem, s>>>(R));
        }
        bytes += V * sk /* flag pre-count */ + rbytes;
        st->levels = L + 1;
        return COUPE_ERR_OK;
    };

    // (the level counts of level 0, the root segments, are written by the
    // root kernel)
    auto finish = [&]() -> int {
        CG_CK(cudaEventRecord(C.ev1, s));
        CG_CK(cudaMemcpyAsync(h_rs, B.rs, sizeof(RunScalars), cudaMemcpyDeviceToHost, s));
        CG_CK(cudaStreamSynchronize(s));
        ++st->host_syncs;
        return COUPE_ERR_OK;
    };
    // Queue levels L.. to the end and wait once.  If a split of level L' needed
    // a third pass, the queued kernels after it did nothing: finish L' with
    // the host's further passes and queue L' + 1.. again.
    uint64_t L = 0;
    bool resume = false;
    while (L < iters) {
        if (resume || tu.sync_levels) {
            const int rc_ = level(L, true, resume);
            resume = false;
            if (rc_ == -1) break;  // a device check failed (h_rs->err)
            if (rc_ != COUPE_ERR_OK) return rc_;
            ++L;
            if (tu.sync_levels || L == iters) {
                if (L == iters) {
                    const int rf = finish();
                    if (rf != COUPE_ERR_OK) return rf;
                }
                continue;
            }
        }
        for (uint64_t l = L; l < iters; ++l) {
            const int rc_ = level(l, false, false);
            if (rc_ != COUPE_ERR_OK) return rc_;
        }
        const int rf = finish();
        if (rf != COUPE_ERR_OK) return rf;
        if (h_rs->err) {
            err_level = (int)iters;  // seen after the queued levels
            break;
        }
        if (!h_rs->stall) break;
        L = h_rs->stall - 1;
        resume = true;
        nspec = std::min(nspec + 1, 3);  // the levels queued again get one more speculative pass
        CG_CK(cudaMemsetAsync(&B.rs->stall, 0, sizeof(uint32_t), s));
    }
    if (h_rs->err && tu.sync_levels) {
        const int rf = finish();  // the stats below read h_rs after the last kernel
        if (rf != COUPE_ERR_OK) return rf;
    }
    C.prof.resolve();
    float ms = 0.f;
    cudaEventElapsedTime(&ms, C.ev0, C.ev1);
    st->device_ms = ms;
    st->splits = h_rs->splits;
    st->split_steps = h_rs->steps_total;
    st->max_split_steps = h_rs->steps_max;
    st->fixed_scale = h_rs->fscale;
    {
        uint64_t lim[4] = {h_rs->wsum_limbs[0], h_rs->wsum_limbs[1], h_rs->wsum_limbs[2], h_rs->wsum_limbs[3]};
        st->root_weight_sum = WL::f64(WL::value(lim, h_rs->fscale));
        st->weight_sum_error_bound = 0.0;
        if (WL::LIMBS > 1) {
            // n quantisation errors of at most 2^(-s-1), then one rounding
            const double a = std::fabs(st->root_weight_sum);
            st->weight_sum_error_bound =
                (double)n * std::ldexp(1.0, -h_rs->fscale - 1) + 0.5 * (std::nextafter(a, INFINITY) - a);
        }
    }
    // refinement passes: the points each scan left for the pass after it
    st->hist_points += h_rs->pass_points;
    bytes += h_rs->pass_points * (sk + sw);
    st->algo_bytes = bytes;
    st->band_points = h_rs->band_points;
    st->weight_rechecks = h_rs->nexactw;
    if (h_rs->err) {
        uint32_t e = h_rs->err;
        if (e & ERR_NONFINITE_WEIGHT) {
            *err = "f64 weights must be finite";
            return COUPE_ERR_BAD_TYPE;
        }
        *err = std::string("device check failed (code ") + std::to_string(e) + ", seen at level " +
               std::to_string(err_level) + " of " + std::to_string(iters) + "; " + std::to_string(h_rs->diag[0]) +
               " " + std::to_string(h_rs->diag[1]) + " " + std::to_string(h_rs->diag[2]) + " " +
               std::to_string(h_rs->diag[3]) + ")";
        return COUPE_ERR_CRASH;
    }
    return COUPE_ERR_OK;
}

template <int D, class KT, class WT>
int run_typed(DevCtx &C, const RunArgs &a, coupe_gpu_stats *st, std::string *err) {
    typedef typename KT::T K;
    NvtxScope run_range(a.nsets > 1 ? "rcb batched run" : "rcb run");
    const Tuning &tu = tuning();
    const uint64_t n = a.n;
    cudaStream_t s = a.stream ? a.stream : C.stream;
    st->points = n;
    if (n == 0) return COUPE_ERR_OK;
    if (n > 0xffffffffull) {
        *err = "more than 2^32 - 1 points";
        return COUPE_ERR_ALLOC;
    }
    const bool multi = a.nsets > 1;
    // Several sets: root segments for the non-empty sets with iter_count > 0,
    // in set order; the deepest set gives the number of levels.
    std::vector<uint32_t> h_root, h_roots;
    std::vector<uint64_t> h_P;
    uint64_t v0 = n, max_iters = a.iter_count;
    if (multi) {
        h_root.assign(a.nsets, ~0u);
        v0 = 0;
        max_iters = 0;
        for (uint64_t k = 0; k < a.nsets; ++k) {
            const uint64_t nk = a.set_off[k + 1] - a.set_off[k];
            if (nk == 0 || a.set_iters[k] == 0) continue;
            h_root[k] = (uint32_t)h_roots.size();
            h_roots.push_back((uint32_t)k);
            h_P.push_back(v0);
            v0 += nk;
            max_iters = std::max<uint64_t>(max_iters, a.set_iters[k]);
        }
        h_P.push_back(v0);
    }
    if (max_iters == 0) {
        // rcb_recurse with iter_count == 0 stores id 0 everywhere (:589-602)
        CG_LAUNCH(KID_FILL, n * 8,
                  k_fill_u64<<<std::max<uint64_t>(1, std::min<uint64_t>((n + 255) / 256, 4096)), 256, 0, s>>>(a.d_part,
                                                                                                            n, 0));
        CG_CK(cudaStreamSynchronize(s));
        return COUPE_ERR_OK;
    }
    const uint64_t iters = max_iters;
    uint64_t scap = 1, tcap = 0;
    bool index_path = false;
    std::vector<uint64_t> smax(iters), vmax(iters);
    if (multi) {
        // level L holds at most min(2^L, n_k) segments of each set deeper
        // than L, and every item of those sets
        for (uint64_t L = 0; L < iters && L < 64; ++L) {
            uint64_t cnt = 0, items = 0;
            for (uint32_t k : h_roots) {
                const uint64_t nk = a.set_off[k + 1] - a.set_off[k];
                if (a.set_iters[k] > L) {
                    cnt += L < 40 ? std::min<uint64_t>(nk, 1ull << L) : nk;
                    items += nk;
                }
            }
            smax[L] = cnt;
            vmax[L] = items;
            scap = std::max(scap, cnt);
            tcap += cnt;
        }
        scap = std::max<uint64_t>(scap, h_roots.size());
        if (iters > (uint64_t)MAX_TRAV_LEVELS || tcap > TRAV_MAX_ENTRIES) {
            *err = "batched run: more than " + std::to_string(MAX_TRAV_LEVELS) + " levels or " +
                   std::to_string(TRAV_MAX_ENTRIES) + " splits";
            return COUPE_ERR_ALLOC;
        }
    } else {
        // segment capacity: a level holds at most min(2^level, n) segments
        scap = iters >= 40 ? n : std::min<uint64_t>(n, 1ull << iters);
        scap = std::max<uint64_t>(scap, 1);
        // Part ids come from a traversal of the recorded splits unless the
        // tree is too large to record; then every reorder carries the input
        // indices.
        for (uint64_t L = 0; L < iters && tcap <= TRAV_MAX_ENTRIES; ++L)
            tcap += L < 40 ? std::min<uint64_t>(n, 1ull << L) : n;
        index_path = tu.force_index_path || iters > (uint64_t)MAX_TRAV_LEVELS || tcap > TRAV_MAX_ENTRIES;
        for (uint64_t L = 0; L < iters; ++L) {
            smax[L] = L < 40 ? std::min<uint64_t>(n, 1ull << L) : n;
            vmax[L] = n;
        }
    }
    const uint64_t hb = std::max<uint64_t>(2 * scap, std::min<uint64_t>(scap * MAX_NB, 1ull << 22));
    // look-back words: one per reorder chunk; a reorder grid never exceeds 8
    // CTAs of BLOCK threads per SM, so this capacity fits every weight type
    const uint64_t lbcap = (uint64_t)C.sms * 8 * (uint64_t)std::max(1, tu.reorder_chunks_per_cta);

    Buffers<D, KT, WT> B;
    Bump dry{nullptr, 0};
    const bool carry = index_path || KT::BAND;
    const uint64_t nsets = multi ? a.nsets : 0;
    const size_t need = B.carve(dry, n, scap, hb, lbcap, index_path, carry, tcap, nsets, iters);
    // 256 bytes of slack: reorder tiles are copied in 16-byte chunks that may
    // end up to 15 bytes past a buffer
    int rc = ensure_workspace(C, need + 256, err);
    if (rc != COUPE_ERR_OK) return rc;
    Bump real{(char *)C.ws, 0};
    B.carve(real, n, scap, hb, lbcap, index_path, carry, tcap, nsets, iters);
    const SetTab sets = B.set_tab(multi ? (uint32_t)a.nsets : 1u);
    RunScalars *h_rs = (RunScalars *)C.h_pinned;

    const int g_stream = std::max<int>(1, std::min<uint64_t>((n + BLOCK - 1) / BLOCK, (uint64_t)C.sms * 8));

    CG_CK(cudaEventRecord(C.ev0, s));
    RunScalars init;
    std::memset(&init, 0, sizeof(init));
    for (int d = 0; d < 3; ++d) {
        init.bbox_min_ord[d] = ord_f64(1.7976931348623157e308);
        init.bbox_max_ord[d] = ord_f64(-1.7976931348623157e308);
    }
    init.min_heap = ~0ull;
    *h_rs = init;
    CG_CK(cudaMemcpyAsync(B.rs, h_rs, sizeof(RunScalars), cudaMemcpyHostToDevice, s));
    if (multi) {
        // the set table (pageable copies: the host vectors are read before
        // the calls return)
        const uint64_t nr = h_roots.size();
        CG_CK(cudaMemcpyAsync(B.set_off, a.set_off, (nsets + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
        CG_CK(cudaMemcpyAsync(B.set_iters, a.set_iters, nsets * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
        CG_CK(cudaMemcpyAsync(B.set_root, h_root.data(), nsets * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
        CG_CK(cudaMemcpyAsync(B.roots, h_roots.data(), nr * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
        CG_CK(cudaMemcpyAsync(B.P[0], h_P.data(), (nr + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
        CG_LAUNCH(KID_ROOT, 0, k_sets_init<<<(unsigned)((nsets + 255) / 256), 256, 0, s>>>(sets));
    }

    Mat M;
    std::memset(&M, 0, sizeof(M));
    M.on = a.has_matrix ? 1 : 0;
    for (int i = 0; i < 9; ++i) M.m[i] = a.matrix[i];
    const uint64_t sk = sizeof(K), sw = sizeof(typename WT::S);
    if (M.on && sizeof(K) == 4 && sets.count <= 1) {
        CG_LAUNCH(KID_CONVERT, n * (D * 8 + D * sk),
                  k_convert<D, KT, true><<<g_stream, BLOCK, 0, s>>>(a.d_points, n, M, B.keys[0][0], B.keys[0][1],
                                                                    B.keys[0][2], B.rs, sets));
    } else {
        CG_LAUNCH(KID_CONVERT, n * (D * 8 + D * sk),
                  k_convert<D, KT><<<g_stream, BLOCK, 0, s>>>(a.d_points, n, M, B.keys[0][0], B.keys[0][1],
                                                              B.keys[0][2], B.rs, sets));
    }
    const typename WT::S *w_in = (const typename WT::S *)a.d_weights;
    if (a.weights_ready) CG_CK(cudaStreamWaitEvent(s, a.weights_ready, 0));
    if (WT::LIMBS > 1) {
        CG_LAUNCH(KID_WABS, n * sw, k_wabs_max<<<g_stream, BLOCK, 0, s>>>((const double *)w_in, n, B.rs, sets));
        if (multi) CG_LAUNCH(KID_WABS, 0, k_set_fs<<<(unsigned)((nsets + 255) / 256), 256, 0, s>>>(sets, B.rs));
    }
    // integer weights: the weight sum also writes a 16-bit copy into w[0]
    // (which level 0 does not otherwise use) for the level loop to read when
    // every weight lies in [0, 2^16)
    uint16_t *c16 = WT::LIMBS == 1 ? (uint16_t *)B.w[0] : nullptr;
    CG_LAUNCH(KID_WSUM, n * sw + (c16 ? n * 2 : 0), k_wsum<WT><<<g_stream, BLOCK, 0, s>>>(w_in, n, B.rs, c16, sets));

    RunSetup R0;
    R0.n = n;
    R0.iters = iters;
    R0.nsets = multi ? (uint32_t)a.nsets : 1u;
    R0.nroots = multi ? (uint32_t)h_roots.size() : 1u;
    R0.v0 = v0;
    R0.index_path = index_path;
    R0.carry = carry;
    R0.M = M;
    R0.s = s;
    R0.h_rs = h_rs;
    R0.g_stream = g_stream;
    R0.lbcap = lbcap;
    R0.smax = std::move(smax);
    R0.vmax = std::move(vmax);
    // algorithmic bytes: the input read and the SoA keys written
    R0.bytes = n * (D * 8 + sw) + n * D * sk + n * sw + (c16 ? n * 2 : 0);  // convert + weight sum
    if (WT::LIMBS > 1) R0.bytes += n * sw;
    if constexpr (WT::LIMBS == 1) {
        CG_CK(cudaMemcpyAsync(h_rs, B.rs, sizeof(RunScalars), cudaMemcpyDeviceToHost, s));
        CG_CK(cudaStreamSynchronize(s));
        ++st->host_syncs;
        if (h_rs->narrow16 == 0) return run_levels<D, KT, WT, WtC16<WT>>(C, a, st, err, B, R0, c16);
    }
    return run_levels<D, KT, WT, WT>(C, a, st, err, B, R0, w_in);
}

template <class KT>
int run_mode(DevCtx &C, const RunArgs &a, coupe_gpu_stats *st, std::string *err) {
    if (a.dim == 2) {
        switch (a.wtype) {
        case 0: return run_typed<2, KT, WtI32>(C, a, st, err);
        case 1: return run_typed<2, KT, WtI64>(C, a, st, err);
        case 2: return run_typed<2, KT, WtF64>(C, a, st, err);
        }
    } else if (a.dim == 3) {
        switch (a.wtype) {
        case 0: return run_typed<3, KT, WtI32>(C, a, st, err);
        case 1: return run_typed<3, KT, WtI64>(C, a, st, err);
        case 2: return run_typed<3, KT, WtF64>(C, a, st, err);
        }
    } else {
        return COUPE_ERR_BAD_DIMENSION;
    }
    *err = "unknown weight type";
    return COUPE_ERR_BAD_TYPE;
}

}  // namespace cg
