"""Replica bookkeeping for `bench.py --gpus N` under torchrun.

A single state vector does not shard without a global-qubit exchange, so N
GPUs run N independent replicas of the workload; the only collective is on
the host (gloo): a barrier around the timed region and the maximum of the
per-rank times.  `value` is then N x (per-replica work) / max time."""
import os


def world():
    return (int(os.environ.get('WORLD_SIZE', '1')), int(os.environ.get('RANK', '0')),
            int(os.environ.get('LOCAL_RANK', '0')))


def init():
    size, rank, local = world()
    if size > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group('gloo')
    return size, rank, local


def barrier():
    size, _, _ = world()
    if size > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(value):
    size, _, _ = world()
    if size == 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t[0])


def aggregate_throughput(work_per_rank, local_seconds):
    """(whole-job throughput, max seconds): every rank did `work_per_rank`."""
    size, _, _ = world()
    t = max_over_ranks(local_seconds)
    return work_per_rank * size / t, t


def finish():
    size, _, _ = world()
    if size > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()
