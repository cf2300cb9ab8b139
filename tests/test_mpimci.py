"""MPIMCI over torch.distributed (gloo, two CPU processes): seeds scattered from a
seed file, results combined with the reference's formula (src/MPIMCI.cpp:85-92),
and the error behaviour of the reference's functions."""
import os
import socket

import numpy as np
import pytest


class FakeMCI:
    """An MCI whose integrate returns fixed per-rank numbers and records its seed."""

    def __init__(self, rank):
        self.rank = rank
        self.seed = None

    def setSeed(self, s):
        self.seed = s

    def getNObsDim(self):
        return 3

    def integrate(self, nmc, find=True, decorr=True):
        r = self.rank
        return np.array([1.0 + r, -2.0 * r, 0.5]), np.array([0.1 * (r + 1), 0.2, 0.3 + r])


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, seedfile, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    from mcintegratorplusplus_gb300 import mpimci
    try:
        out = {}
        try:
            mpimci.integrate(FakeMCI(rank), 10)
        except RuntimeError as e:
            out["before_init"] = str(e)
        assert mpimci.init("gloo") == rank
        try:
            mpimci.init("gloo")
        except RuntimeError as e:
            out["twice"] = str(e)
        out["size"] = mpimci.size()
        m = FakeMCI(rank)
        mpimci.setSeed(m, seedfile, offset=1)
        out["seed"] = m.seed
        try:
            mpimci.setSeed(m, seedfile, offset=4)
        except RuntimeError as e:
            out["too_few"] = str(e)
        avg, err = mpimci.integrate(m, 100)
        out["avg"], out["err"] = avg.tolist(), err.tolist()
        mpimci.finalize()
        q.put((rank, out))
    except Exception as e:  # report instead of hanging the parent
        q.put((rank, {"error": repr(e)}))


def test_mpimci_two_processes(tmp_path):
    import torch.multiprocessing as mp
    seedfile = tmp_path / "rseed.txt"
    seedfile.write_text("11 22 33\n44 55\n")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, str(seedfile), q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    for r in (0, 1):
        assert "error" not in res[r], res[r]
        assert res[r]["before_init"] == "MPI not initialized!"
        assert res[r]["twice"] == "MPI already initialized!"
        assert res[r]["size"] == 2
        assert "enough seeds" in res[r]["too_few"]
    assert (res[0]["seed"], res[1]["seed"]) == (22, 33)  # offset 1 skips the first seed
    a = [FakeMCI(r).integrate(1) for r in (0, 1)]
    exp_avg = (a[0][0] + a[1][0]) / 2
    exp_err = np.sqrt(a[0][1] ** 2 + a[1][1] ** 2) / 2
    for r in (0, 1):
        np.testing.assert_allclose(res[r]["avg"], exp_avg, rtol=1e-15)
        np.testing.assert_allclose(res[r]["err"], exp_err, rtol=1e-15)
