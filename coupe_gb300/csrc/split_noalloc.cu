// coupe_gpu_split_noalloc: a stable split of one part of device-resident
// points by a cut on one axis, for callers that must not allocate device
// memory once they are running.
//
// It is a variant of the level reorder (k_reorder) for a single segment whose
// left count is not known in advance:
//   k_split_count  one CTA per chunk counts the chunk's items with
//                  point[coord] < cut into the scratch's per-chunk counts;
//   k_split_move   one CTA per chunk reads all chunk counts (its exclusive
//                  prefix and the total), then walks the chunk in tiles staged
//                  by cp.async (double buffered), ranks each tile with warp
//                  ballots and one warp scan, and writes the tile's left and
//                  right items as two coalesced runs of whole points.
// No kernel waits on another CTA.  The only scratch is g_split_scratch, a
// file-scope device array of SPLIT_SCRATCH_WORDS words; nothing is allocated
// with cudaMalloc, cudaMallocAsync, cudaHostAlloc or a library allocator, and
// no stream or event is created.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <mutex>

#include "kernels.cuh"
#include "split_noalloc.h"

namespace cg {

namespace {

constexpr uint32_t SPLIT_MAX_CHUNKS = 1024;  // per-chunk counts the scratch holds
constexpr int SCR_TOTAL = 0;                 // word: left items of the part (written by chunk 0)
constexpr int SCR_ERR = 1;                   // word: ERR_* bits, cleared by every call
constexpr int SCR_CNT = 8;                   // words [8, 8 + SPLIT_MAX_CHUNKS): left items per chunk
constexpr int SPLIT_SCRATCH_WORDS = SCR_CNT + SPLIT_MAX_CHUNKS;  // 8256 bytes
constexpr int MAX_DEVICES = 64;

static __device__ __align__(256) uint64_t g_split_scratch[SPLIT_SCRATCH_WORDS];

// point[coord] < cut with IEEE semantics (false when either is NaN, -0 == +0),
// computed on order-preserving integer codes.
__device__ __forceinline__ bool split_left(double x, uint64_t cut_code) {
    return KeyF64::lt(KeyF64::from_f64_bits((uint64_t)__double_as_longlong(x)), cut_code);
}

template <int D>
__global__ void __launch_bounds__(BLOCK) k_split_count(const double *__restrict__ pts, uint64_t n, uint64_t chunk,
                                                       int coord, uint64_t cut_code, uint64_t *scr) {
    __shared__ uint64_t sh[33];
    const uint64_t t = blockIdx.x;
    const uint64_t c0 = t * chunk, c1 = min(n, c0 + chunk);
    uint64_t c = 0;
    for (uint64_t i = c0 + threadIdx.x; i < c1; i += BLOCK) c += split_left(pts[i * D + coord], cut_code) ? 1 : 0;
    uint64_t total;
    block_exscan_u64(c, sh, total);
    if (threadIdx.x == 0) scr[SCR_CNT + t] = total;
}

template <int D, class WS>
__host__ __device__ constexpr size_t split_tile_bytes() {
    return (size_t)R_TILE * (D * sizeof(double) + sizeof(WS));
}

template <int D, class WS>
__host__ __device__ constexpr size_t split_smem() {
    return 2 * split_tile_bytes<D, WS>() + (size_t)R_TILE * sizeof(uint16_t);
}

template <int D, class WS>
__global__ void __launch_bounds__(BLOCK, 2) k_split_move(const double *__restrict__ pts, const WS *__restrict__ w,
                                                         uint64_t n, uint64_t chunk, uint32_t nchunks, int coord,
                                                         uint64_t cut_code, double *__restrict__ out_pts,
                                                         WS *__restrict__ out_w, uint64_t *scr) {
    extern __shared__ __align__(16) unsigned char dsm[];
    constexpr size_t TB = split_tile_bytes<D, WS>();
    uint16_t *perm = (uint16_t *)(dsm + 2 * TB);  // run slot -> item of the tile
    __shared__ uint32_t s_cnt[R_ITEMS * NWARPS];
    __shared__ uint64_t sh[33];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    auto tile_p = [&](int buf) { return (double *)(dsm + buf * TB); };
    auto tile_w = [&](int buf) { return (WS *)(dsm + buf * TB + (size_t)R_TILE * D * sizeof(double)); };
    auto prefetch = [&](uint64_t ts, uint64_t te, int buf) {
        const uint32_t cnt = (uint32_t)(te - ts);
        double *tp = tile_p(buf);
        WS *tw = tile_w(buf);
        const double *gp = pts + ts * D;
        for (uint32_t q = threadIdx.x; q < cnt * D; q += BLOCK) cp_async<8>(tp + q, gp + q);
        for (uint32_t q = threadIdx.x; q < cnt; q += BLOCK) cp_async<sizeof(WS)>(tw + q, w + ts + q);
        cp_async_commit();
    };

    const uint64_t t = blockIdx.x;
    const uint64_t c0 = t * chunk, c1 = min(n, c0 + chunk);
    prefetch(c0, min(c0 + R_TILE, c1), 0);  // overlaps the prefix below
    uint64_t pre = 0, tot = 0;
    for (uint32_t i = threadIdx.x; i < nchunks; i += BLOCK) {
        const uint64_t v = scr[SCR_CNT + i];
        tot += v;
        if (i < t) pre += v;
    }
    uint64_t prefix, total;
    block_exscan_u64(pre, sh, prefix);
    block_exscan_u64(tot, sh, total);
    if (t == 0 && threadIdx.x == 0) scr[SCR_TOTAL] = total;
    uint64_t lpos = prefix;                 // next left slot of this chunk
    uint64_t rpos = total + (c0 - prefix);  // next right slot of this chunk
    int buf = 0;
    for (uint64_t ts = c0; ts < c1; ts += R_TILE) {
        const uint64_t te = min(ts + R_TILE, c1);
        if (te < c1) {
            prefetch(te, min(te + R_TILE, c1), buf ^ 1);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();  // this tile's copies are visible to every thread
        const uint32_t tcount = (uint32_t)(te - ts);
        const double *tp = tile_p(buf);
        const WS *tw = tile_w(buf);
        bool fl[R_ITEMS];
        uint32_t bal[R_ITEMS];
#pragma unroll
        for (int i = 0; i < R_ITEMS; ++i) {
            const uint32_t li = i * BLOCK + threadIdx.x;
            fl[i] = li < tcount && split_left(tp[li * D + coord], cut_code);
            bal[i] = __ballot_sync(0xffffffffu, fl[i]);
            if (lane == 0) s_cnt[i * NWARPS + warp] = __popc(bal[i]);
        }
        __syncthreads();
        if (warp == 0) {
            // exclusive scan of R_ITEMS * NWARPS counts in (row, warp) order
            constexpr int PER = (R_ITEMS * NWARPS + 31) / 32;
            uint32_t v[PER], sum = 0;
#pragma unroll
            for (int j = 0; j < PER; ++j) {
                const int idx = lane * PER + j;
                v[j] = idx < R_ITEMS * NWARPS ? s_cnt[idx] : 0;
                sum += v[j];
            }
            uint32_t inc = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += u;
            }
            uint32_t run = inc - sum;
#pragma unroll
            for (int j = 0; j < PER; ++j) {
                const int idx = lane * PER + j;
                if (idx < R_ITEMS * NWARPS) s_cnt[idx] = run;
                run += v[j];
            }
            if (lane == 31) sh[0] = inc;
        }
        __syncthreads();
        const uint32_t tile_left = (uint32_t)sh[0];
#pragma unroll
        for (int i = 0; i < R_ITEMS; ++i) {
            const uint32_t li = i * BLOCK + threadIdx.x;
            if (li < tcount) {
                const uint32_t before = s_cnt[i * NWARPS + warp] + __popc(bal[i] & ((1u << lane) - 1));
                const uint32_t slot = fl[i] ? before : tile_left + (li - before);
                if (slot < tcount)
                    perm[slot] = (uint16_t)li;
                else
                    atomicOr((unsigned int *)&scr[SCR_ERR], ERR_TILE_PERM);
            }
        }
        __syncthreads();
        // the left run, then the right run: thread q writes double q of a run
        const bool ok = lpos + tile_left <= total && rpos + (tcount - tile_left) <= n;
        if (!ok) {
            if (threadIdx.x == 0) atomicOr((unsigned int *)&scr[SCR_ERR], ERR_SCATTER_BOUNDS);
        } else {
            double *lo = out_pts + lpos * D, *ro = out_pts + rpos * D;
            for (uint32_t q = threadIdx.x; q < tile_left * D; q += BLOCK) {
                const uint32_t k = q / D, j = q - k * D, src = perm[k];
                if (src < tcount) lo[q] = tp[src * D + j];
            }
            for (uint32_t q = threadIdx.x; q < (tcount - tile_left) * D; q += BLOCK) {
                const uint32_t k = q / D, j = q - k * D, src = perm[tile_left + k];
                if (src < tcount) ro[q] = tp[src * D + j];
            }
            for (uint32_t k = threadIdx.x; k < tcount; k += BLOCK) {
                const uint32_t src = perm[k];
                if (src >= tcount) {
                    atomicOr((unsigned int *)&scr[SCR_ERR], ERR_TILE_PERM);
                    continue;
                }
                if (k < tile_left)
                    out_w[lpos + k] = tw[src];
                else
                    out_w[rpos + (k - tile_left)] = tw[src];
            }
        }
        lpos += tile_left;
        rpos += tcount - tile_left;
        __syncthreads();  // the buffer and perm are free again
        buf ^= 1;
    }
}

// Per-device set-up, done once with that device current: the scratch's
// device address and the move kernels' shared-memory attribute.
struct SplitDevice {
    bool ready = false;
    uint64_t *scr = nullptr;
    int grid_cap = 0;  // most chunks a call uses (resident move CTAs, <= SPLIT_MAX_CHUNKS)
};
SplitDevice g_split_dev[MAX_DEVICES];
std::mutex g_split_mu;

template <int D, class WS>
cudaError_t set_move_attr() {
    return cudaFuncSetAttribute((const void *)k_split_move<D, WS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)split_smem<D, WS>());
}

int split_setup(SplitDevice **out, const char **msg) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) {
        *msg = "no current CUDA device (or its ordinal is above 63)";
        return COUPE_ERR_CRASH;
    }
    std::lock_guard<std::mutex> lock(g_split_mu);
    SplitDevice &S = g_split_dev[dev];
    if (!S.ready) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_split_scratch) != cudaSuccess || p == nullptr) {
            *msg = "cudaGetSymbolAddress of the split scratch failed";
            return COUPE_ERR_CRASH;
        }
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) {
            *msg = "cudaDeviceGetAttribute(multiProcessorCount) failed";
            return COUPE_ERR_CRASH;
        }
        if (set_move_attr<2, int32_t>() != cudaSuccess || set_move_attr<2, int64_t>() != cudaSuccess ||
            set_move_attr<2, double>() != cudaSuccess || set_move_attr<3, int32_t>() != cudaSuccess ||
            set_move_attr<3, int64_t>() != cudaSuccess || set_move_attr<3, double>() != cudaSuccess) {
            *msg = "cudaFuncSetAttribute(MaxDynamicSharedMemorySize) of the split kernels failed";
            return COUPE_ERR_CRASH;
        }
        int per = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, (const void *)k_split_move<3, double>, BLOCK,
                                                          split_smem<3, double>()) != cudaSuccess ||
            per < 1)
            per = 1;
        S.scr = (uint64_t *)p;
        S.grid_cap = (int)std::min<int64_t>((int64_t)sms * per, SPLIT_MAX_CHUNKS);
        S.ready = true;
    }
    *out = &S;
    return COUPE_ERR_OK;
}

template <int D, class WS>
void launch_split(const SplitDevice &S, const double *pts, const void *w, uint64_t n, uint64_t chunk,
                  uint32_t nchunks, int coord, uint64_t cut_code, double *out_pts, void *out_w, cudaStream_t s) {
    k_split_count<D><<<nchunks, BLOCK, 0, s>>>(pts, n, chunk, coord, cut_code, S.scr);
    k_split_move<D, WS><<<nchunks, BLOCK, split_smem<D, WS>(), s>>>(pts, (const WS *)w, n, chunk, nchunks, coord,
                                                                   cut_code, out_pts, (WS *)out_w, S.scr);
}

}  // namespace

int split_noalloc(uint64_t n, uint64_t dimension, const double *d_points, int weight_type, const void *d_weights,
                  uint64_t coord, double cut, double *d_out_points, void *d_out_weights, uint64_t *n_left,
                  void *stream, const char **msg) {
    *msg = "";
    if (dimension != 2 && dimension != 3) return COUPE_ERR_BAD_DIMENSION;
    if (weight_type < COUPE_INT || weight_type > COUPE_DOUBLE) {
        *msg = "unknown weight type";
        return COUPE_ERR_BAD_TYPE;
    }
    if (coord >= dimension) {
        *msg = "coord must be below dimension";
        return COUPE_ERR_BAD_TYPE;
    }
    if (n > SPLIT_MAX_POINTS) {
        *msg = "more than 2^32 - 1 points: coupe_gpu_split_noalloc splits at most 4294967295 points per call";
        return COUPE_ERR_ALLOC;
    }
    if (!n_left) {
        *msg = "NULL n_left";
        return COUPE_ERR_BAD_TYPE;
    }
    if (n == 0) {
        *n_left = 0;
        return COUPE_ERR_OK;
    }
    if (!d_points || !d_weights || !d_out_points || !d_out_weights) {
        *msg = "NULL input or output pointer";
        return COUPE_ERR_BAD_TYPE;
    }
    if (cudaPeekAtLastError() != cudaSuccess) {
        // not ours: an error the caller's earlier work left pending
        *msg = "a CUDA error from earlier work on this thread is pending (cudaPeekAtLastError); nothing was launched";
        return COUPE_ERR_CRASH;
    }
    SplitDevice *S = nullptr;
    int rc = split_setup(&S, msg);
    if (rc != COUPE_ERR_OK) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    // chunks grow with n, so a call never needs more than grid_cap counts
    uint64_t chunk = std::max<uint64_t>(R_TILE, (n + S->grid_cap - 1) / (uint64_t)S->grid_cap);
    chunk = (chunk + R_TILE - 1) / R_TILE * R_TILE;
    const uint64_t nchunks = (n + chunk - 1) / chunk;
    if (nchunks > SPLIT_MAX_CHUNKS) {
        *msg = "internal: chunk count above the scratch capacity";
        return COUPE_ERR_CRASH;
    }
    const uint64_t cut_code = KeyF64::from_f64(cut);
    // the header (left total, error bits) must start at zero; the counts are
    // all written by k_split_count before k_split_move reads them
    if (cudaMemsetAsync(S->scr, 0, SCR_CNT * sizeof(uint64_t), s) != cudaSuccess) {
        *msg = "cudaMemsetAsync of the split scratch header failed";
        return COUPE_ERR_CRASH;
    }
    const int c = (int)coord;
    const uint32_t nc = (uint32_t)nchunks;
    if (dimension == 2) {
        if (weight_type == COUPE_INT)
            launch_split<2, int32_t>(*S, d_points, d_weights, n, chunk, nc, c, cut_code, d_out_points, d_out_weights, s);
        else if (weight_type == COUPE_INT64)
            launch_split<2, int64_t>(*S, d_points, d_weights, n, chunk, nc, c, cut_code, d_out_points, d_out_weights, s);
        else
            launch_split<2, double>(*S, d_points, d_weights, n, chunk, nc, c, cut_code, d_out_points, d_out_weights, s);
    } else {
        if (weight_type == COUPE_INT)
            launch_split<3, int32_t>(*S, d_points, d_weights, n, chunk, nc, c, cut_code, d_out_points, d_out_weights, s);
        else if (weight_type == COUPE_INT64)
            launch_split<3, int64_t>(*S, d_points, d_weights, n, chunk, nc, c, cut_code, d_out_points, d_out_weights, s);
        else
            launch_split<3, double>(*S, d_points, d_weights, n, chunk, nc, c, cut_code, d_out_points, d_out_weights, s);
    }
    if (cudaGetLastError() != cudaSuccess) {
        *msg = "launch of the split kernels failed";
        return COUPE_ERR_CRASH;
    }
    uint64_t hdr[2] = {0, 0};
    if (cudaMemcpyAsync(hdr, S->scr, sizeof(hdr), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        *msg = "device to host copy of the split result failed";
        return COUPE_ERR_CRASH;
    }
    if (hdr[SCR_ERR]) {
        *msg = (hdr[SCR_ERR] & ERR_SCATTER_BOUNDS) ? "device check failed: split run out of bounds"
                                                   : "device check failed: tile permutation out of range";
        return COUPE_ERR_CRASH;
    }
    *n_left = hdr[SCR_TOTAL];
    return COUPE_ERR_OK;
}

}  // namespace cg
