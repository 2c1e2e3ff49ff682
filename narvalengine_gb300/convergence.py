"""Converged reference images and time-to-relMSE of the plain integrator.

relMSE(x, ref) = mean over pixels and channels of (x - ref)^2 / (ref^2 + 1e-2).

The reference image is the mean of many samples per pixel, each path's radiance converted
to FP64 and summed on the device in sample order (ne_render_accumulate), in chunks of
samples so the per-path buffer stays bounded. It is rendered with its own seed, so its
samples are independent of the images measured against it. The reference integrator can
return a non-finite radiance on rare paths (a zero in a pdf denominator); those paths are
dropped from every accumulated image and counted (`dropped_paths`).

Time-to-relMSE renders progressively, doubling the samples per pixel (1, 2, 4, ...), until
the image's relMSE against the reference is at or below the target, and reports the
cumulative device time of the samples rendered so far.

    python -m narvalengine_gb300.convergence --scene medium_c2 --ref-spp 65536 --target 1e-3
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

REF_SEED = 0x5EED_0F_2EF
EPS = 1e-2


def relmse(x: np.ndarray, ref: np.ndarray, eps: float = EPS) -> float:
    x = np.asarray(x, np.float64)
    ref = np.asarray(ref, np.float64)
    return float(np.mean((x - ref) ** 2 / (ref * ref + eps)))


def _accumulate(scene, acc, seed: int, first: int, count: int, chunk: int, dropped: list) -> float:
    """Adds samples [first, first + count) to the device accumulator; device milliseconds."""
    from . import NE_RENDER_DROP_NONFINITE, NE_RENDER_OUT_DEVICE, render_params
    ms = 0.0
    done = 0
    while done < count:
        n = min(chunk, count - done)
        scene.ctx.record(0)
        st = scene.accumulate(acc.data_ptr(), render_params(seed=seed, spp=n, sample_offset=first + done,
                                                            flags=NE_RENDER_OUT_DEVICE | NE_RENDER_DROP_NONFINITE))
        scene.ctx.record(1)
        ms += scene.ctx.elapsed_ms(0, 1)
        dropped[0] += st["dropped_paths"]
        done += n
    return ms


def reference_image(scene, spp: int, seed: int = REF_SEED, chunk: int = 256, info: dict | None = None):
    """FP64 mean of `spp` samples per pixel (H, W, 3), and the device milliseconds it took."""
    import torch
    H, W = scene.host.height, scene.host.width
    acc = torch.zeros((H, W, 3), dtype=torch.float64, device=f"cuda:{scene.ctx.device}")
    dropped = [0]
    ms = _accumulate(scene, acc, seed, 0, spp, chunk, dropped)
    if info is not None:
        info["dropped_paths"] = dropped[0]
    return (acc / float(spp)).cpu().numpy(), ms


def time_to_relmse(scene, ref: np.ndarray, target: float = 1e-3, seed: int = 0, max_spp: int = 1 << 16,
                   chunk: int = 256) -> dict:
    """Progressive render (samples added in powers of two) until relMSE <= target.

    `ms` is the cumulative device time of all samples up to that point, the time a
    progressive renderer needs to reach the target."""
    import torch
    H, W = scene.host.height, scene.host.width
    acc = torch.zeros((H, W, 3), dtype=torch.float64, device=f"cuda:{scene.ctx.device}")
    curve = []
    have, spp, ms = 0, 1, 0.0
    hit = None
    dropped = [0]
    while spp <= max_spp:
        ms += _accumulate(scene, acc, seed, have, spp - have, chunk, dropped)
        have = spp
        e = relmse((acc / float(spp)).cpu().numpy(), ref)
        curve.append({"spp": spp, "relmse": e, "ms": ms})
        if e <= target:
            hit = curve[-1]
            break
        spp *= 2
    return {"target": target, "reached": hit is not None, "spp": hit["spp"] if hit else None,
            "ms": hit["ms"] if hit else None, "dropped_paths": dropped[0], "curve": curve}


def main(argv=None):
    import narvalengine_gb300 as ne
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--scene", default="medium_c2")
    ap.add_argument("--ref-spp", type=int, default=65536)
    ap.add_argument("--chunk", type=int, default=256)
    ap.add_argument("--target", type=float, default=1e-3)
    ap.add_argument("--resolution", type=int, nargs=2, default=None, help="override width height")
    ap.add_argument("--save", default=None, help="write the reference image (.npy)")
    args = ap.parse_args(argv)
    path = args.scene if args.scene.endswith(".json") else os.path.join(ne.SCENES_DIR, args.scene + ".json")
    if args.resolution:
        d = json.load(open(path))
        d["renderer"]["resolution"] = list(args.resolution)
        host = ne.SceneHost.from_string(json.dumps(d), os.path.dirname(path))
    else:
        host = ne.SceneHost.from_json(path)
    ctx = ne.Context(0)
    scene = ctx.upload(host)
    t0 = time.time()
    info = {}
    ref, ref_ms = reference_image(scene, args.ref_spp, chunk=args.chunk, info=info)
    if args.save:
        np.save(args.save, ref)
    res = time_to_relmse(scene, ref, args.target, chunk=args.chunk)
    out = {"scene": os.path.basename(path), "resolution": [host.width, host.height], "ref_spp": args.ref_spp,
           "ref_paths": host.width * host.height * args.ref_spp, "ref_device_ms": ref_ms,
           "ref_wall_s": time.time() - t0, "ref_dropped_paths": info["dropped_paths"], "relmse_eps": EPS, **res}
    print(json.dumps(out))
    scene.close()
    ctx.close()


if __name__ == "__main__":
    main()
