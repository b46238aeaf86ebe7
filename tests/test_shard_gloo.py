"""The multi-rank path on CPU ranks (gloo, world size 2): shot sharding,
the one gradient/misfit reduction, and a rank that fails before the
reduction (the other rank sees an error, it does not hang)."""
import datetime
import os
import socket

import numpy as np
import pytest

from libemmi_mgfd_gb300.shard import ShardedObjective, allreduce_sum, shots_of_rank


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _partial(shots, shape=(2, 7, 9, 11)):
    """A rank's share: per-shot gradients (seeded by the shot number) summed
    over its shots, and the per-shot misfits summed."""
    g = np.zeros(shape, np.float32)
    f = np.zeros(1, np.float32)
    for s in shots:
        rng = np.random.default_rng(1000 + s)
        g += rng.standard_normal(shape).astype(np.float32)
        f += np.float32(rng.uniform(0.5, 2.0))
    return g, f


def _rank(rank, world, port, nshots, fail_rank, out):
    import torch.distributed as D
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    D.init_process_group("gloo", rank=rank, world_size=world,
                         timeout=datetime.timedelta(seconds=10))
    try:
        mine = shots_of_rank(nshots, rank, world)
        if rank == fail_rank:
            raise RuntimeError("rank failed before the reduction")
        g, f = _partial(mine)
        g, f = allreduce_sum([g, f], D)
        np.savez(os.path.join(out, f"r{rank}.npz"), g=g, f=f, shots=np.array(mine))
    except Exception as e:  # reported to the parent through the file system
        with open(os.path.join(out, f"r{rank}.err"), "w") as fh:
            fh.write(repr(e))
    finally:
        try:
            D.destroy_process_group()
        except Exception:
            pass


def _run(world, nshots, fail_rank, tmp_path):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, world, port, nshots, fail_rank, str(tmp_path)))
          for r in range(world)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert not p.is_alive(), "a rank hung"
    return tmp_path


@pytest.mark.parametrize("nshots,world", [(25, 2), (5, 2), (7, 3), (1, 1), (25, 8)])
def test_shots_cover_every_shot_once(nshots, world):
    got = [s for r in range(world) for s in shots_of_rank(nshots, r, world)]
    assert got == list(range(1, nshots + 1))
    sizes = [len(shots_of_rank(nshots, r, world)) for r in range(world)]
    assert max(sizes) - min(sizes) <= 1


def test_shots_list_is_validated():
    assert shots_of_rank(9, 1, 2, shots=[3, 5, 7]) == [7]
    with pytest.raises(ValueError):
        shots_of_rank(4, 0, 1, shots=[5])


def test_gradient_and_misfit_sum_over_two_gloo_ranks(tmp_path):
    _run(2, 5, -1, tmp_path)
    g_all, f_all = _partial(range(1, 6))
    seen = []
    for r in range(2):
        assert not (tmp_path / f"r{r}.err").exists(), (tmp_path / f"r{r}.err").read_text()
        d = np.load(tmp_path / f"r{r}.npz")
        seen += list(d["shots"])
        # float32 sums in a different order than one rank's: a few ulps
        np.testing.assert_allclose(d["g"], g_all, rtol=1e-5, atol=1e-5)
        np.testing.assert_allclose(d["f"], f_all, rtol=1e-6)
    assert sorted(seen) == [1, 2, 3, 4, 5]


def test_a_failed_rank_makes_the_reduction_fail_not_hang(tmp_path):
    _run(2, 4, 1, tmp_path)
    assert (tmp_path / "r1.err").exists()
    # rank 0 either sees the peer's exit as an error or times out: no result
    assert (tmp_path / "r0.err").exists()
    assert not (tmp_path / "r0.npz").exists()


class _FakeFg:
    """Stands in for gpu.Fg on CPU ranks: each shot's misfit, gradient and
    pseudo-Hessian are seeded by its shot number and scaled by the model."""

    def __init__(self, shots, shape=(2, 5, 6, 7)):
        self.shots, self.shape = list(shots), shape

    def eval(self, model):
        fc, g, h = [], np.zeros(self.shape, np.float32), np.zeros(self.shape, np.float32)
        for s in self.shots:
            rng = np.random.default_rng(2000 + s)
            fc.append(np.float32(model * rng.uniform(1.0, 3.0)))
            g += np.float32(model) * rng.standard_normal(self.shape).astype(np.float32)
            h += rng.uniform(0.0, 1.0, self.shape).astype(np.float32)
        return np.array(fc, np.float32), g, h


def _objective_rank(rank, world, port, nshots, out):
    import torch.distributed as D
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    D.init_process_group("gloo", rank=rank, world_size=world,
                         timeout=datetime.timedelta(seconds=10))
    try:
        obj = ShardedObjective(_FakeFg(shots_of_rank(nshots, rank, world)), D)
        f, g, h = obj(1.5)
        np.savez(os.path.join(out, f"o{rank}.npz"), f=f, g=g, h=h)
    finally:
        D.destroy_process_group()


def test_sharded_objective_sums_over_two_gloo_ranks(tmp_path):
    """The per-rank objective (this rank's shots in one evaluation, then one
    reduction) gives every rank the all-shot totals."""
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    port = _free_port()
    ps = [ctx.Process(target=_objective_rank, args=(r, 2, port, 5, str(tmp_path)))
          for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert not p.is_alive() and p.exitcode == 0
    f1, g1, h1 = ShardedObjective(_FakeFg(range(1, 6)))(1.5)
    for r in range(2):
        d = np.load(tmp_path / f"o{r}.npz")
        assert abs(float(d["f"]) - f1) <= 1e-6 * abs(f1)
        np.testing.assert_allclose(d["g"], g1, rtol=1e-5, atol=1e-5)
        np.testing.assert_allclose(d["h"], h1, rtol=1e-5, atol=1e-5)
