"""Multi-rank path on CPU: world-size-2 gloo ranks shard a batch of
independent structures with no data-path collective and reduce only the
bookkeeping, which must equal the single-rank result."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, root, out):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, here)
    import conftest  # noqa: F401  (import paths)
    import torch
    import torch.distributed as dist
    from fbgpu import batch, synth
    from oracle import oracle as orc
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    structs = synth.batch_structures(8)
    path = synth.fdata_dir_for("batch256", root=root)
    fd = orc.Fdata(path, [14, 6])
    pairs = 0
    for k in batch.shard(len(structs), rank, world):
        st = structs[k]
        pairs += orc.System(fd, st.ratom, st.imass, st.lattice).neighbors().npairs
    t = torch.tensor([pairs], dtype=torch.int64)
    dist.all_reduce(t)
    if rank == 0:
        np.save(out, t.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_shard_matches_serial(fdata_root, tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    from fbgpu import synth
    from oracle import oracle as orc
    out = str(tmp_path / "total.npy")
    mp.start_processes(_worker, args=(2, _free_port(), fdata_root, out), nprocs=2, start_method="spawn")
    structs = synth.batch_structures(8)
    fd = orc.Fdata(synth.fdata_dir_for("batch256", root=fdata_root), [14, 6])
    serial = sum(orc.System(fd, s.ratom, s.imass, s.lattice).neighbors().npairs for s in structs)
    assert int(np.load(out)[0]) == serial


def test_shard_covers_each_item_once():
    from fbgpu import batch
    for world in (1, 2, 3, 8):
        got = sorted(i for r in range(world) for i in batch.shard(37, r, world))
        assert got == list(range(37))
    with pytest.raises(ValueError):
        batch.shard(4, 2, 2)


def test_weighted_shard_balances_the_batch():
    """Longest-first sharding of the 256-structure batch by its three-center
    work estimate: every item once, the same partition on every rank, and
    the largest rank load within the greedy rule's bound (at most the mean
    load plus the largest item), well below the round-robin split's."""
    from fbgpu import batch, synth
    structs = synth.batch_structures(256)
    w = np.array([batch.work_estimate(s.ratom, s.lattice) for s in structs])
    for world in (2, 4, 8):
        parts = [batch.shard(len(w), r, world, weights=w) for r in range(world)]
        assert sorted(i for p in parts for i in p) == list(range(len(w)))
        loads = np.array([w[p].sum() for p in parts])
        assert loads.max() <= w.sum() / world + w.max() + 1e-9
        rr = np.array([w[batch.shard(len(w), r, world)].sum() for r in range(world)])
        assert loads.max() <= rr.max()
        assert loads.max() / loads.mean() < 1.02


def test_work_estimate_tracks_triplets(fdata_root):
    """The estimate orders structures like their actual triplet counts."""
    from fbgpu import batch, synth
    from oracle import oracle as orc
    structs = synth.batch_structures(12)
    fd = orc.Fdata(synth.fdata_dir_for("batch256", root=fdata_root), [14, 6])
    est = np.array([batch.work_estimate(s.ratom, s.lattice) for s in structs])
    trip = np.array([orc.System(fd, s.ratom, s.imass, s.lattice).neighbors().ntrip for s in structs])
    ratio = trip / est
    assert ratio.max() / ratio.min() < 1.5
