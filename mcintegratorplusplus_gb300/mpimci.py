"""MPIMCI: one MCI per process, results combined across processes.

Mirrors the reference's MPIMCI namespace (include/mci/MPIMCI.hpp:11-30,
src/MPIMCI.cpp) over torch.distributed instead of MPI: each process (one per GPU,
launched by torchrun or any launcher that sets RANK / WORLD_SIZE / MASTER_ADDR /
MASTER_PORT) integrates its own MCI and the averages and errors are reduced with
the MPIMCI formula (src/MPIMCI.cpp:85-92): average = mean over processes,
error = sqrt(sum of squared errors) / nprocesses.  The chains of one process are
already combined the same way by MCI.integrate, so a run over P processes of
n chains each gives the estimate of P * n chains.

The functions take any object with the MCI methods they call (integrate,
getNObsDim, setSeed), so the host logic runs on CPU processes too.
"""
import os

import numpy as np

__all__ = ["init", "myrank", "size", "setSeed", "integrate", "finalize"]


def _dist():
    import torch.distributed as dist
    return dist


def init(backend=None):
    """MPIMCI::init (src/MPIMCI.cpp:24-34): start the process group, return this rank.

    backend: "nccl" when CUDA is available, else "gloo" (default)."""
    dist = _dist()
    if dist.is_initialized():
        raise RuntimeError("MPI already initialized!")
    if backend is None:
        import torch
        backend = "nccl" if torch.cuda.is_available() else "gloo"
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group(backend)
    return myrank()


def _check():
    dist = _dist()
    if not dist.is_initialized():
        raise RuntimeError("MPI not initialized!")
    return dist


def myrank():
    return _check().get_rank()


def size():
    return _check().get_world_size()


def setSeed(mci, filename, offset=0):
    """MPIMCI::setSeed (src/MPIMCI.cpp:38-65): rank 0 reads `offset` seeds to skip and
    then one seed per process from a whitespace-separated file; every process gets
    its own."""
    dist = _check()
    nranks, rank = dist.get_world_size(), dist.get_rank()
    payload = [None]
    if rank == 0:
        try:
            with open(filename) as f:
                words = f.read().split()
        except OSError:
            payload = [RuntimeError("Random seed file could not be found.")]
        else:
            if offset > len(words):
                payload = [RuntimeError("Chosen seed offset is already larger than the number of seeds in seed file.")]
            elif offset + nranks > len(words):
                payload = [RuntimeError("Seed file doesn't provide enough seeds for the chosen number of ranks and offset.")]
            else:
                payload = [[int(w) for w in words[offset:offset + nranks]]]
    dist.broadcast_object_list(payload, src=0)
    if isinstance(payload[0], Exception):
        raise payload[0]
    mci.setSeed(payload[0][rank])


def integrate(mci, Nmc, doFindMRT2step=True, doDecorrelation=True):
    """MPIMCI::integrate (src/MPIMCI.cpp:68-92): every process integrates, then
    average = sum(average) / P and error = sqrt(sum(error^2)) / P on every process.
    Returns (average, error) as numpy arrays."""
    import torch
    dist = _check()
    nranks = dist.get_world_size()
    avg, err = mci.integrate(Nmc, doFindMRT2step, doDecorrelation)
    avg = np.asarray(avg, dtype=np.float64)
    err = np.asarray(err, dtype=np.float64)
    backend = dist.get_backend()
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    a = torch.tensor(avg, dtype=torch.float64, device=dev)
    e2 = torch.tensor(err * err, dtype=torch.float64, device=dev)
    dist.all_reduce(a, op=dist.ReduceOp.SUM)
    dist.all_reduce(e2, op=dist.ReduceOp.SUM)
    return a.cpu().numpy() / nranks, np.sqrt(e2.cpu().numpy()) / nranks


def finalize():
    """MPIMCI::finalize (src/MPIMCI.cpp:95-104)."""
    dist = _dist()
    if not dist.is_initialized():
        raise RuntimeError("MPI not initialized!")
    dist.destroy_process_group()
