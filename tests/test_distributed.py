"""Multi-rank layouts of Rcb on CPU ranks (gloo, world size 2 and 4).

The GPU pool of this build runs one GPU per process, so the protocol of
coupe_gb300/distributed.py is tested here with host restatements of the
per-rank computations (the fold of one bisection step over a rank's points,
recursive_bisection.rs:478-503, and the Rcb of a subtree from its state,
:575-642); the part ids are compared with the oracle's single-process run.
"""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from coupe_gb300 import distributed as D  # noqa: E402

F32 = np.float32


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


# -- host restatements of the per-rank computations (test doubles) ---------

def fold_int(k, w, t):
    left = k < t
    d = (k[~left] - t).astype(F32)
    d = d[np.isfinite(d) | (d < 0)]
    nd = F32(d.min()) if len(d) else F32(np.inf)
    return int(left.sum()), int(np.sum(w[left], dtype=np.int64)), nd


def make_fold_f64(state):
    def fold(k, w, t):
        left = k < t
        d = (k[~left] - t).astype(F32)
        nd = F32(d.min()) if len(d) else F32(np.inf)
        return int(left.sum()), D.fixed_limbs(w[left], state.s), nd
    return fold


def make_local_rcb(fold, fw, state=None):
    """coupe's rcb_recurse from a given segment state (REF32)."""
    def wval(x):
        return D.limbs_value(x, state.s) if fw else D._wrap64(int(x))

    def local_rcb(keys, w, iters, tol, heap, coord, bmin, bmax, total):
        ids = np.zeros(len(w), dtype=np.uint64)
        Dm = keys.shape[1]

        def rec(rows, it, h, c, bmn, bmx, tot):
            if len(rows) == 0:
                return
            if it == 0:
                ids[rows] = h
                return
            k, ww = keys[rows, c], w[rows]
            mn, mx, prev = F32(bmn[c]), F32(bmx[c]), None
            while True:
                t = F32((mn + mx) / F32(2.0))
                cnt, wl, nd = fold(k, ww, t)
                wl = wval(wl)
                if not np.isfinite(nd) and nd > 0:
                    if prev == cnt:
                        all_left, sp, wl_out = True, mx, tot
                        break
                    mx, prev = t, cnt
                    continue
                ideal = float(tot) / 2.0
                with np.errstate(divide="ignore", invalid="ignore"):
                    imb = abs((float(wl) - ideal) / ideal)
                if cnt == prev or mx <= F32(t + nd) or imb <= tol:
                    all_left, sp, wl_out = False, t, wl
                    break
                prev = cnt
                wr = (tot - wl) if fw else D._wrap64(tot - wl)
                if wl < wr:
                    mn = t
                else:
                    mx = t
            left = np.ones(len(rows), dtype=bool) if all_left else k < sp
            lmax, rmin = list(bmx), list(bmn)
            lmax[c] = float(sp)
            rmin[c] = float(sp)
            wr = (tot - wl_out) if fw else D._wrap64(tot - wl_out)
            nc = (c + 1) % Dm
            rec(rows[left], it - 1, 2 * h + 1, nc, bmn, lmax, wl_out)
            rec(rows[~left], it - 1, 2 * h + 2, nc, rmin, bmx, wr)

        rec(np.arange(len(w)), iters, heap, coord, list(bmin), list(bmax), total)
        return ids
    return local_rcb


def _worker(rank, world, port, case, out_path):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rng = np.random.default_rng(case["seed"])
        n, dim = case["n"], case["dim"]
        pts = rng.random((n, dim)) * 10.0
        if case["fw"]:
            w = rng.lognormal(0.0, 1.0, size=n)
        else:
            w = rng.integers(1, 100, size=n, dtype=np.int64)
        # a random split of the points over the ranks (not contiguous)
        owner = np.random.default_rng(99).integers(0, world, size=n)
        mine = np.nonzero(owner == rank)[0]
        keys = pts[mine].astype(F32)
        bmin = torch.from_numpy(pts[mine].min(axis=0) if len(mine) else np.full(dim, np.inf))
        bmax = torch.from_numpy(pts[mine].max(axis=0) if len(mine) else np.full(dim, -np.inf))
        dist.all_reduce(bmin, op=dist.ReduceOp.MIN)
        dist.all_reduce(bmax, op=dist.ReduceOp.MAX)

        class Holder:
            s = 0
        state = Holder()
        fold = make_fold_f64(state) if case["fw"] else fold_int
        if case["fw"]:
            # the restated fold needs the run's fixed-point scale: that of the
            # largest |w| over all ranks and the global count
            amax = float(np.max(np.abs(w[mine]))) if len(mine) else 0.0
            t = torch.tensor([amax], dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            state.s = D.fixed_scale(float(t.item()), n)
        algo = D.SingleSetRcb(dist.group.WORLD, fold, make_local_rcb(fold, case["fw"], state), case["fw"])
        g, ids = algo.partition(keys, w[mine], mine.astype(np.int64), n, case["iters"], case["tol"],
                                      (bmin.numpy().tolist(), bmax.numpy().tolist()))
        # gather everything on rank 0
        objs = [None] * world
        dist.all_gather_object(objs, (g.tolist(), ids.tolist()))
        if rank == 0:
            full = np.zeros(n, dtype=np.uint64)
            seen = np.zeros(n, dtype=bool)
            for gg, ii in objs:
                full[np.asarray(gg, dtype=np.int64)] = np.asarray(ii, dtype=np.uint64)
                seen[np.asarray(gg, dtype=np.int64)] = True
            assert seen.all()
            np.save(out_path, full)
            np.save(out_path + ".pts.npy", pts)
            np.save(out_path + ".w.npy", w)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("case", [
    dict(seed=1, n=20000, dim=3, fw=False, iters=6, tol=0.01, world=2),
    dict(seed=2, n=15000, dim=2, fw=False, iters=5, tol=0.05, world=4),
    dict(seed=3, n=3000, dim=3, fw=True, iters=4, tol=0.01, world=2),
])
def test_single_set_over_ranks_equals_oracle(oracle_mod, tmp_path, case):
    out = str(tmp_path / "ids.npy")
    mp.start_processes(_worker, args=(case["world"], _free_port(), case, out), nprocs=case["world"],
                       start_method="spawn")
    got = np.load(out)
    pts, w = np.load(out + ".pts.npy"), np.load(out + ".w.npy")
    want, _ = oracle_mod.rcb(pts, w, case["iters"], case["tol"], fsum=oracle_mod.FSUM_FIXED)
    assert (got == want).all(), int((got != want).sum())


def test_fixed_point_sums_are_bit_identical_over_any_split(oracle_mod):
    """The all-reduced limb sums of any split of the weights equal the sums
    of the whole, and round to the oracle's fixed-point total."""
    rng = np.random.default_rng(5)
    w = rng.lognormal(0.0, 2.0, size=5000)
    w[::7] *= -1
    s = D.fixed_scale(float(np.abs(w).max()), len(w))
    assert s == oracle_mod.fixed_scale(w)
    whole = D.fixed_limbs(w, s)
    for parts in (2, 3, 8):
        cut = np.sort(rng.choice(len(w), parts - 1, replace=False))
        pieces = np.split(rng.permutation(w), cut)
        acc = sum(D.fixed_limbs(p, s) for p in pieces)
        # limb sums differ in their carries but the 128-bit totals agree
        tot = lambda L: sum(int(L[l]) << (32 * l) for l in range(4)) & ((1 << 128) - 1)  # noqa: E731
        assert tot(acc) == tot(whole)
    assert D.limbs_value(whole, s) == oracle_mod.fixed_sum(w, s)


def test_shard_sets_balances_and_covers():
    rng = np.random.default_rng(3)
    sizes = rng.integers(1000, 1_000_000, size=500)
    for world in (1, 2, 3, 8):
        plan = D.shard_sets(sizes, world)
        assert sorted(k for p in plan for k in p) == list(range(len(sizes)))
        loads = [int(sizes[p].sum()) for p in plan]
        assert max(loads) - min(loads) <= int(sizes.max())  # greedy bound
        assert plan == D.shard_sets(sizes, world)  # every rank computes the same plan


def _batched_worker(rank, world, port, out_path):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import sys
        sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
        import oracle
        rng = np.random.default_rng(11)
        sizes = rng.integers(50, 3000, size=40)
        off = np.zeros(len(sizes) + 1, dtype=np.uint64)
        np.cumsum(sizes, out=off[1:])
        pts = rng.random((int(off[-1]), 2))
        w = rng.integers(1, 10, size=len(pts), dtype=np.int64)
        its = rng.integers(1, 7, size=len(sizes)).astype(np.uint32)

        def cpu_partition(p, ww, o, it, tol, mode):
            return oracle.rcb_sets(p, ww, o, it, tol)
        rows, ids = D.rcb_batched_sharded(pts, w, off, its, 0.02, rank, world, partition=cpu_partition)
        objs = [None] * world
        dist.all_gather_object(objs, (rows.tolist(), ids.tolist()))
        if rank == 0:
            full = np.zeros(len(pts), dtype=np.uint64)
            for r, i in objs:
                full[np.asarray(r, dtype=np.int64)] = np.asarray(i, dtype=np.uint64)
            want = oracle.rcb_sets(pts, w, off, its, 0.02)
            np.save(out_path, (full == want).astype(np.int8))
    finally:
        dist.destroy_process_group()


def test_batched_sharded_over_ranks(tmp_path):
    out = str(tmp_path / "ok.npy")
    mp.start_processes(_batched_worker, args=(2, _free_port(), out), nprocs=2, start_method="spawn")
    assert np.load(out).all()


def _failing_worker(rank, world, port, out_dir):
    """Rank 1's fold raises on its first call; rank 0 must see its next
    collective end with an error (the peer is gone) instead of waiting."""
    import datetime
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=10))
    status = "finished"
    try:
        rng = np.random.default_rng(5)
        n = 4000
        pts = rng.random((n, 2))
        w = rng.integers(1, 100, size=n, dtype=np.int64)
        mine = np.arange(rank, n, world)

        def fold(k, ww, t):
            if rank == 1:
                raise RuntimeError("injected failure in rank 1's fold")
            return fold_int(k, ww, t)
        algo = D.SingleSetRcb(dist.group.WORLD, fold, make_local_rcb(fold_int, False), False)
        algo.partition(pts[mine].astype(F32), w[mine], mine.astype(np.int64), n, 4, 0.01,
                       (pts.min(axis=0).tolist(), pts.max(axis=0).tolist()))
    except Exception as e:  # recorded for the test, then the rank leaves
        status = "error: %s: %s" % (type(e).__name__, str(e)[:200])
    finally:
        with open(os.path.join(out_dir, "rank%d.txt" % rank), "w") as f:
            f.write(status)
        if rank == 1:
            os._exit(0)  # leave without a clean shutdown, as a crashed rank does
        try:
            dist.destroy_process_group()
        except Exception:
            pass


def test_failing_rank_ends_the_others_collectives(tmp_path):
    """A rank that fails between collectives (host-side failure, no GPU):
    its error is its own, and the surviving rank's next all-reduce ends with
    an error within the group's timeout instead of hanging."""
    mp.start_processes(_failing_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    r1 = open(tmp_path / "rank1.txt").read()
    r0 = open(tmp_path / "rank0.txt").read()
    assert r1.startswith("error: RuntimeError: injected failure"), r1
    assert r0.startswith("error:"), r0
