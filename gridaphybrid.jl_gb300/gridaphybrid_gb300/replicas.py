"""Independent replicas on several GPUs of one node.

The hybridization path is not sharded across GPUs here.  Under torchrun,
every rank runs the whole workload on its own GPU (LOCAL_RANK) and nothing is
exchanged on the data path.  The process group exists only for measurement:
a barrier on both sides of the timed region, then the maximum elapsed time
over ranks.  NCCL is used when CUDA is available, gloo otherwise.
"""
import os


def world():
    """(rank, world_size, local_rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend=None):
    """Initialises the process group when WORLD_SIZE > 1; returns (rank, world, local_rank)."""
    rank, size, local = world()
    if size > 1:
        import torch
        import torch.distributed as dist
        if not dist.is_initialized():
            if backend is None:
                backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(local)
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group(backend=backend, rank=rank, world_size=size)
    return rank, size, local


def _active():
    try:
        import torch.distributed as dist
        return dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1
    except ImportError:
        return False


def barrier():
    if _active():
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(value):
    """The maximum of a float over all ranks (the value itself on one rank)."""
    if not _active():
        return float(value)
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank, seconds_per_rank):
    """Whole-job throughput: units over all ranks / max elapsed time over ranks."""
    _, size, _ = world() if _active() else (0, 1, 0)
    tmax = max_over_ranks(seconds_per_rank)
    return size * units_per_rank / tmax, tmax


def finalize():
    if _active():
        import torch.distributed as dist
        dist.destroy_process_group()
