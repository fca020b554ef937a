"""Rcb across several GPUs: one process per GPU (torch.distributed ranks).

coupe itself is single-process: rayon forks the bisection tree into
independent subtrees (coupe/src/algorithms/recursive_bisection.rs:618-641),
and each split's loop folds and reduces one segment (:478-520).  Across GPUs
the same structure gives two layouts:

* Batched form (many independent point sets): the sets are dealt to the
  ranks, balanced by their point counts (`shard_sets`), and every rank runs
  the batched entry point on its own sets.  No collective touches the data
  path; part ids stay with the rank that owns the set.
  (`rcb_batched_sharded`.)

* One large set spread over G = 2^g ranks (`SingleSetRcb`): the top g tree
  levels need every rank's points.  Each step of a split's loop reduces a
  per-segment tuple over the ranks — (count left, weight left, nearest
  distance) — with one all-reduce for all segments of the level: integer
  weights as wrapping int64 sums, f64 weights as the 128-bit fixed point of
  the engine in four 32-bit limbs (integer sums: identical whatever the
  split of the points over the ranks), the nearest distance as a minimum.
  Every rank then replays coupe's decision on the same totals.  After g
  levels subtree j of the 2^g belongs to rank j: one all-to-all moves the
  points there, and the remaining levels run on each rank alone from the
  subtree's state (box, weight sum, heap id, axis).  Part ids are shifted by
  the smallest heap id over all ranks (:698-702).

  The per-rank computations (the fold of one step over a rank's points and
  the Rcb of a subtree) are callables: this module holds the protocol only.
  This build's GPU pool runs one GPU per process, so the protocol is tested
  on CPU ranks (gloo) with host restatements of those callables.
"""
import math

import numpy as np

# ---------------------------------------------------------------------------
# Batched form
# ---------------------------------------------------------------------------


def shard_sets(set_sizes, world):
    """Deals sets to `world` ranks, largest first, each to the rank with the
    fewest points so far (ties: the lowest rank).  Returns one ascending list
    of set numbers per rank; deterministic, so every rank computes the same
    plan without communicating."""
    sizes = np.asarray(set_sizes, dtype=np.int64)
    order = sorted(range(len(sizes)), key=lambda k: (-int(sizes[k]), k))
    load = [0] * world
    plan = [[] for _ in range(world)]
    for k in order:
        r = min(range(world), key=lambda i: (load[i], i))
        plan[r].append(k)
        load[r] += int(sizes[k])
    return [sorted(p) for p in plan]


def local_sets(points, weights, set_offsets, iter_counts, sets):
    """The rows of the given sets, concatenated in set order, with the set
    table of the concatenation and each row's global index."""
    off = np.asarray(set_offsets, dtype=np.int64)
    idx = [np.arange(off[k], off[k + 1], dtype=np.int64) for k in sets]
    rows = np.concatenate(idx) if idx else np.zeros(0, dtype=np.int64)
    sizes = np.array([off[k + 1] - off[k] for k in sets], dtype=np.uint64)
    loff = np.zeros(len(sets) + 1, dtype=np.uint64)
    np.cumsum(sizes, out=loff[1:])
    its = np.array([iter_counts[k] for k in sets], dtype=np.uint32)
    return points[rows], weights[rows], loff, its, rows


def rcb_batched_sharded(points, weights, set_offsets, iter_counts, tolerance, rank, world, partition=None,
                        mode="ref32"):
    """This rank's share of a batched Rcb: (global row indices, part ids).

    `partition(points, weights, set_offsets, iter_counts, tolerance, mode)`
    returns the ids of a batched run over the rank's sets; by default the
    library's batched entry point on the rank's current GPU.  Ids are those
    of each set alone, so no collective is needed; gather them if one rank
    needs them all."""
    sizes = np.diff(np.asarray(set_offsets, dtype=np.int64))
    plan = shard_sets(sizes, world)
    p, w, loff, its, rows = local_sets(points, weights, set_offsets, iter_counts, plan[rank])
    if partition is None:
        partition = _gpu_batched
    ids = partition(p, w, loff, its, tolerance, mode)
    return rows, np.asarray(ids, dtype=np.uint64)


def _gpu_batched(points, weights, set_offsets, iter_counts, tolerance, mode):
    import torch

    from . import rcb_batched_device
    dev = torch.device("cuda", torch.cuda.current_device())
    d_p = torch.from_numpy(np.ascontiguousarray(points)).to(dev)
    d_w = torch.from_numpy(np.ascontiguousarray(weights)).to(dev)
    d_o = torch.empty(len(points), dtype=torch.int64, device=dev)
    rcb_batched_device(d_o, d_p, d_w, set_offsets, iter_counts, tolerance, mode=mode)
    return d_o.cpu().numpy().view(np.uint64)


# ---------------------------------------------------------------------------
# 128-bit fixed-point weights in 32-bit limbs (the engine's order-independent
# f64 sums, coupe_gb300/csrc/common.cuh)
# ---------------------------------------------------------------------------

def fixed_scale(amax, n):
    """s = 126 - e - ceil(log2 n) for 2^(e-1) <= amax < 2^e (0 if amax is 0)."""
    if not amax > 0.0:
        return 0
    _, e = math.frexp(amax)
    return 126 - e - (max(int(n) - 1, 0)).bit_length()


def fixed_limbs(w, s):
    """Sum of round_half_even(w_i 2^s) as four int64 sums of 32-bit chunks of
    the two's-complement 128-bit values (exact for fewer than 2^31 terms)."""
    w = np.asarray(w, dtype=np.float64)
    out = np.zeros(4, dtype=np.int64)
    mask = (1 << 32) - 1
    for x in w.tolist():
        if x == 0.0:
            continue
        m, e = math.frexp(abs(x))
        mi = int(m * (1 << 53))         # exact 53-bit significand
        sh = e - 53 + s
        if sh >= 0:
            q = mi << sh
        else:
            r = -sh
            q = mi >> r if r < 64 else 0
            rem = mi - (q << r) if r < 64 else mi
            half = 1 << (r - 1)
            if r < 64 and (rem > half or (rem == half and (q & 1))):
                q += 1
        if x < 0:
            q = (1 << 128) - q
        for l in range(4):
            out[l] += (q >> (32 * l)) & mask
    return out


def limbs_value(limbs, s):
    """The f64 value (round half to even) of a limb sum: sum / 2^s."""
    Q = sum(int(limbs[l]) << (32 * l) for l in range(4)) & ((1 << 128) - 1)
    if Q >> 127:
        Q -= 1 << 128
    if Q == 0:
        return 0.0
    neg = Q < 0
    a = -Q if neg else Q
    hb = a.bit_length() - 1
    if hb > 52:
        sh = hb - 52
        m = a >> sh
        rem = a - (m << sh)
        half = 1 << (sh - 1)
        if rem > half or (rem == half and (m & 1)):
            m += 1
        v = math.ldexp(float(m), sh - s)
    else:
        v = math.ldexp(float(a), -s)
    return -v if neg else v


# ---------------------------------------------------------------------------
# One large set over G ranks
# ---------------------------------------------------------------------------

_INF32 = np.float32(np.inf)


class _Seg:
    """A segment of one of the top levels: this rank's rows of it and the
    state of coupe's split loop (recursive_bisection.rs:456-573)."""

    def __init__(self, heap, coord, bmin, bmax, total, rows):
        self.heap, self.coord = heap, coord
        self.bmin, self.bmax = list(bmin), list(bmax)
        self.total = total          # weight sum (int wrapping or f64)
        self.rows = rows            # this rank's rows
        self.mn = np.float32(bmin[coord])
        self.mx = np.float32(bmax[coord])
        self.prev = None            # prev_count_left (usize::MAX first)
        self.done = False
        self.split_pos = None
        self.wl = None
        self.all_left = False


def _wrap64(v):
    v &= (1 << 64) - 1
    return v - (1 << 64) if v >> 63 else v


class SingleSetRcb:
    """coupe's Rcb of one point set whose points are spread over the ranks of
    `group` (G = 2^g ranks).  REF32 arithmetic (f32 keys and cuts).

    fold(keys_c, w, t) -> (count_left, weight_left, nearest) over this rank's
    rows of a segment: weight_left an int (integer weights) or limb sums
    (f64 weights, see fixed_limbs), nearest the smallest f32 key - t over
    keys >= t (+inf if none).
    local_rcb(keys, w, iter_count, tol, heap, coord, bmin, bmax, total) ->
    heap ids (un-shifted) of a subtree run alone from that state."""

    def __init__(self, group, fold, local_rcb, float_weights=False):
        import torch.distributed as dist
        self.dist = dist
        self.group = group
        self.G = dist.get_world_size(group)
        self.rank = dist.get_rank(group)
        if self.G & (self.G - 1):
            raise ValueError("the number of ranks must be a power of two")
        self.g = self.G.bit_length() - 1
        self.fold = fold
        self.local_rcb = local_rcb
        self.fw = float_weights

    # -- collectives ------------------------------------------------------
    def _allreduce(self, arr, op):
        import torch
        t = torch.from_numpy(np.ascontiguousarray(arr))
        self.dist.all_reduce(t, op=op, group=self.group)
        return t.numpy()

    def partition(self, keys, weights, gidx, n_global, iter_count, tol, bbox):
        """keys: (n_local, D) f32 keys of this rank's points; gidx their global
        indices; bbox (bmin, bmax) of all points (f64, from an all-reduce of
        the ranks' boxes).  Returns (global indices, part ids) of the points
        this rank holds at the end (its subtree)."""
        import torch.distributed as dist
        D = keys.shape[1]
        w = weights
        if self.fw:
            amax = float(np.max(np.abs(w))) if len(w) else 0.0
            amax = float(self._allreduce(np.array([amax]), dist.ReduceOp.MAX)[0])
            self.s = fixed_scale(amax, n_global)
            total = self._allreduce(fixed_limbs(w, self.s), dist.ReduceOp.SUM)
            total_v = limbs_value(total, self.s)
        else:
            total_v = _wrap64(int(self._allreduce(np.array([int(np.sum(w, dtype=np.int64))], dtype=np.int64),
                                                  dist.ReduceOp.SUM)[0]))
        top = min(self.g, iter_count)
        segs = [_Seg(0, 0, bbox[0], bbox[1], total_v, np.arange(len(w)))]
        for level in range(top):
            segs = self._level(segs, keys, w, tol)
            segs = self._children(segs, keys, D)
        # subtree j (heap ids at depth `top`, in order) belongs to rank j
        return self._exchange_and_finish(segs, keys, w, gidx, iter_count - top, tol, top)

    def _level(self, segs, keys, w, tol):
        import torch.distributed as dist
        active = [s for s in segs if s.rows is not None]
        while True:
            live = [s for s in active if not s.done]
            if not live:
                return segs
            S = len(live)
            cnt = np.zeros(S, dtype=np.int64)
            wl = np.zeros((S, 4), dtype=np.int64) if self.fw else np.zeros(S, dtype=np.int64)
            near = np.full(S, _INF32, dtype=np.float32)
            ts = []
            for i, s in enumerate(live):
                t = np.float32((s.mn + s.mx) / np.float32(2.0))  # recursive_bisection.rs:472
                ts.append(t)
                c, wv, nd = self.fold(keys[s.rows, s.coord], w[s.rows], t)
                cnt[i] = c
                if self.fw:
                    wl[i] = wv
                else:
                    wl[i] = np.int64(_wrap64(int(wv)))
                near[i] = nd
            # one all-reduce of the level's tuples (sums), one of the nearest distances
            cnt = self._allreduce(cnt, dist.ReduceOp.SUM)
            wl = self._allreduce(wl, dist.ReduceOp.SUM)
            near = self._allreduce(near, dist.ReduceOp.MIN)
            for i, s in enumerate(live):
                wv = limbs_value(wl[i], self.s) if self.fw else _wrap64(int(wl[i]))
                self._step(s, ts[i], int(cnt[i]), wv, np.float32(near[i]), tol)

    def _step(self, s, t, count, wl, nd, tol):
        """One iteration of coupe's split loop on the all-reduced totals
        (recursive_bisection.rs:522-571)."""
        if not np.isfinite(nd) and nd > 0:  # no item right of t
            if s.prev == count:
                s.done, s.all_left, s.split_pos, s.wl = True, True, s.mx, s.total
                return
            s.mx = t
            s.prev = count
            return
        total = s.total
        ideal = float(total) / 2.0
        with np.errstate(divide="ignore", invalid="ignore"):
            imb = abs((float(wl) - ideal) / ideal)
        stop = count == s.prev or s.mx <= np.float32(t + nd) or imb <= tol
        if stop:
            s.done, s.split_pos, s.wl = True, t, wl
            return
        s.prev = count
        wr = (total - wl) if self.fw else _wrap64(total - wl)
        if wl < wr:
            s.mn = t
        else:
            s.mx = t

    def _children(self, segs, keys, D):
        out = []
        for s in segs:
            if s.rows is None:
                out += [_Seg.__new__(_Seg), _Seg.__new__(_Seg)]
                for c in out[-2:]:
                    c.rows = None
                continue
            k = keys[s.rows, s.coord]
            left = np.ones(len(s.rows), dtype=bool) if s.all_left else (k < np.float32(s.split_pos))
            lmax, rmin = list(s.bmax), list(s.bmin)
            lmax[s.coord] = float(s.split_pos)
            rmin[s.coord] = float(s.split_pos)
            nc = (s.coord + 1) % D
            wr = (s.total - s.wl) if self.fw else _wrap64(s.total - s.wl)
            out.append(_Seg(2 * s.heap + 1, nc, s.bmin, lmax, s.wl, s.rows[left]))
            out.append(_Seg(2 * s.heap + 2, nc, rmin, s.bmax, wr, s.rows[~left]))
        # coupe drops empty children (recursive_bisection.rs:586-588): a
        # child empty on every rank is dropped here
        import torch.distributed as dist
        sizes = np.array([0 if c.rows is None else len(c.rows) for c in out], dtype=np.int64)
        sizes = self._allreduce(sizes, dist.ReduceOp.SUM)
        for c, sz in zip(out, sizes):
            if sz == 0:
                c.rows = None
        return out

    def _exchange_and_finish(self, segs, keys, w, gidx, rest, tol, top):
        """The exchange plan: subtree j (the j-th segment of depth `top`, heap
        order) goes to rank j * G / 2^top (rank j when top == g).  One
        all-to-all moves each row with its subtree number; each rank then
        runs its subtrees alone."""
        import torch
        import torch.distributed as dist
        G, r = self.G, self.rank
        nsub = len(segs)
        owner = [j * G // nsub for j in range(nsub)]
        send_rows = [[] for _ in range(G)]
        send_sub = [[] for _ in range(G)]
        for j, sg in enumerate(segs):
            if sg.rows is not None and len(sg.rows):
                send_rows[owner[j]].append(sg.rows)
                send_sub[owner[j]].append(np.full(len(sg.rows), j, dtype=np.int64))
        cat = lambda xs: np.concatenate(xs) if xs else np.zeros(0, dtype=np.int64)  # noqa: E731
        order = cat([cat(x) for x in send_rows])
        sub = cat([cat(x) for x in send_sub])
        counts = torch.tensor([sum(len(a) for a in x) for x in send_rows], dtype=torch.int64)
        recv_counts = torch.empty(G, dtype=torch.int64)
        dist.all_to_all_single(recv_counts, counts, group=self.group)
        sc, rc = counts.tolist(), recv_counts.tolist()

        def xchg(arr):
            t = torch.from_numpy(np.ascontiguousarray(arr))
            out = torch.empty((sum(rc),) + tuple(t.shape[1:]), dtype=t.dtype)
            dist.all_to_all_single(out, t, output_split_sizes=rc, input_split_sizes=sc, group=self.group)
            return out.numpy()
        k_in, w_in, g_in, s_in = xchg(keys[order]), xchg(w[order]), xchg(gidx[order]), xchg(sub)
        ids = np.zeros(len(g_in), dtype=np.uint64)
        for j, sg in enumerate(segs):
            if owner[j] != r or sg.rows is None:
                continue
            m = s_in == j
            if m.any():
                ids[m] = self.local_rcb(k_in[m], w_in[m], rest, tol, sg.heap, sg.coord, sg.bmin, sg.bmax, sg.total)
        # part_ids -= min(part_ids) over all ranks (recursive_bisection.rs:698-702)
        mn = int(ids.min()) if len(ids) else (1 << 62)
        mn = int(self._allreduce(np.array([mn], dtype=np.int64), dist.ReduceOp.MIN)[0])
        return g_in, ids - np.uint64(mn)
