"""The multi-rank exchange of the filter stage with gloo ranks on the CPU
(world size 2 and 3): sharding of starts and slabs, the all-to-all
redistribution and back, the sharded Rayleigh-Ritz step against the
single-process result, and the fault cases (a rank that raises before a
collective, a rank that never arrives) ending in ShardError on the others
instead of a hang."""
import os
import socket

import numpy as np
import pytest

from filterbse_gb300.shard import ShardError, ShardedRitz, ritz, slab, start_shard

DV = 0.125


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _problem(nstart=6, L=301, seed=5):
    """A small Hermitian H with a known spectrum and filtered-like states."""
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.normal(size=(L, L)) + 1j * rng.normal(size=(L, L)))
    ev = np.linspace(-1.0, 2.0, L)
    H = (Q * ev) @ Q.conj().T
    low = Q[:, :8] @ (rng.normal(size=(8, nstart)) + 1j * rng.normal(size=(8, nstart)))
    psi = (low + 1e-3 * (rng.normal(size=(L, nstart)) + 1j * rng.normal(size=(L, nstart)))).T
    return H, psi, ev


def _worker(rank, world, port, mode, q):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    try:
        from datetime import timedelta
        dist.init_process_group("gloo", rank=rank, world_size=world, timeout=timedelta(seconds=20))
        H, psi, _ = _problem()
        mine = start_shard(len(psi), world, rank)
        local = torch.from_numpy(psi[mine].copy())
        hlocal = torch.from_numpy((H @ psi[mine].T).T.copy())
        ex = ShardedRitz(deadline=3.0)
        if mode == "roundtrip":
            s = ex.to_slabs(local)
            back = ex.from_slabs(s, ex.counts(len(mine)))
            q.put((rank, "ok", bool(torch.equal(back, local)), s.shape))
        elif mode == "ritz":
            e, sg, vec = ritz(ex, local, hlocal, DV)
            q.put((rank, "ok", e, sg))
        elif mode == "raise":
            if rank == 1:
                raise RuntimeError("rank 1 fails before the exchange")
            ritz(ex, local, hlocal, DV)
            q.put((rank, "ok", None, None))
        dist.destroy_process_group()
    except ShardError as e:
        q.put((rank, "shard_error", str(e), None))
    except Exception as e:  # the planted failure of rank 1, or anything unexpected
        q.put((rank, "error", repr(e), None))


def _spawn(world, mode):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, world, port, mode, q)) for r in range(world)]
    for p in ps:
        p.start()
    out = [q.get(timeout=120) for _ in ps]
    for p in ps:
        p.join(timeout=60)
        if p.is_alive():
            p.kill()
    return sorted(out, key=lambda t: t[0])


def test_shards_cover_everything():
    for world in (1, 2, 3, 5):
        got = np.sort(np.concatenate([start_shard(17, world, r) for r in range(world)]))
        assert np.array_equal(got, np.arange(17))
        spans = [slab(1001, world, r) for r in range(world)]
        assert spans[0][0] == 0 and spans[-1][1] == 1001
        assert all(spans[i][1] == spans[i + 1][0] for i in range(world - 1))
        assert max(h - l for l, h in spans) - min(h - l for l, h in spans) <= 1


@pytest.mark.parametrize("world", [2, 3])
def test_slab_roundtrip(world):
    out = _spawn(world, "roundtrip")
    assert all(o[1] == "ok" and o[2] for o in out), out


def test_sharded_ritz_matches_single_process():
    H, psi, ev = _problem()
    # single process reference: the same step on all states
    a = psi.T  # columns = states
    G = DV * a.conj().T @ a
    M = DV * a.conj().T @ (H @ a)
    lam, V = np.linalg.eigh(G)
    X = V / np.sqrt(lam)
    e_ref = np.linalg.eigvalsh(X.conj().T @ M @ X)
    out = _spawn(2, "ritz")
    for rank, status, e, sg in out:
        assert status == "ok", (rank, e)
        assert np.allclose(e, e_ref, atol=1e-10)
        # the states are noisy mixtures of the 8 lowest eigenvectors: residuals
        # are small but not zero, the same on every rank
        assert np.all(sg >= 0) and np.all(sg < 0.1)
    assert np.array_equal(out[0][2], out[1][2])  # replicated eigensolve: identical on every rank


def test_failed_rank_is_reported_not_hung():
    out = _spawn(2, "raise")
    assert out[1][1] == "error" and "rank 1 fails" in out[1][2]
    assert out[0][1] == "shard_error" and "[1]" in out[0][2]
