"""Multi-rank sharding on the CPU (gloo, world size 2).

Camera paths are independent, so N GPUs split a render by sample ranges: rank r renders
samples [r*spp, (r+1)*spp) of every pixel, with no collective on the data path (bench.py).
Here two gloo ranks render their ranges of a small scene with the CPU oracle, use bench.py's
barrier and max helpers, and sum their images once at the end; the mean over ranks must
equal one render of all 2*spp samples.
"""
import os
import socket

import numpy as np
import pytest

from conftest import ROOT, scene_path

torch = pytest.importorskip("torch")


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def small_scene_json():
    import json
    d = json.load(open(scene_path("cornell_c1")))
    d["renderer"]["resolution"] = [24, 16]
    d["renderer"]["spp"] = 2
    return json.dumps(d)


def worker(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import sys
    sys.path.insert(0, ROOT)
    import bench
    import narvalengine_gb300 as ne
    from oracle import oracle as orc
    d = bench.Dist(world, "gloo")
    o = orc.OracleScene.from_json(text=small_scene_json())
    spp = o.spp
    img, secs = o.render(ne.render_params(seed=4, spp=spp, sample_offset=rank * spp), threads=1)
    d.barrier()
    slowest = d.max(float(rank + 1))
    t = torch.from_numpy(img.astype(np.float64))
    d.dist.all_reduce(t)
    if rank == 0:
        np.save(os.path.join(out_dir, "sum.npy"), t.numpy())
        np.save(os.path.join(out_dir, "max.npy"), np.array([slowest]))
    d.close()


def test_two_ranks_split_samples(tmp_path, built):
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(worker, args=(world, free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    total = np.load(tmp_path / "sum.npy")
    assert np.load(tmp_path / "max.npy")[0] == 2.0
    import narvalengine_gb300 as ne
    from oracle import oracle as orc
    o = orc.OracleScene.from_json(text=small_scene_json())
    full, _ = o.render(ne.render_params(seed=4, spp=2 * o.spp), threads=1)
    assert np.allclose(total / world, full, rtol=1e-5, atol=1e-6)
