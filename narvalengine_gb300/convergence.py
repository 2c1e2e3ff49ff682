"""Converged reference images and time-to-relMSE of the plain integrator.

relMSE(x, ref) = mean over pixels and channels of (x - ref)^2 / (ref^2 + 1e-2).

The reference image is the mean of many samples per pixel, each path's radiance converted
to FP64 and summed on the device in sample order (ne_render_accumulate), in chunks of
samples so the per-path buffer stays bounded. It is rendered with its own seed, so its
samples are independent of the images measured against it. The reference integrator
returns a NaN radiance on rare medium paths (HG::sample, materials/Medium.h:109, takes
sqrt(1 - cos^2) without clamping, which is NaN when cos rounds past +-1; about 1.3e-7 of
the medium scene's paths); those paths are dropped from every accumulated image and
counted (`dropped_paths`).

Time-to-relMSE renders progressively, measuring relMSE whenever the sample count has grown
by about 10% (16, 32, 48, ... samples per pixel), until the image's relMSE against the
reference is at or below the target, and reports the cumulative device time of the samples
rendered so far.

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


def checkpoints(first: int, max_spp: int, step: float = 1.1):
    """Sample counts at which relMSE is measured: from `first`, growing by about 10% each."""
    out, s = [], first
    while s <= max_spp:
        out.append(s)
        s = max(s + first, int(round(s * step / first)) * first)
    return out


def time_to_relmse(scene, ref: np.ndarray, target: float = 1e-3, seed: int = 0, max_spp: int = 1 << 16,
                   chunk: int = 256, first: int = 16) -> dict:
    """Progressive render until relMSE <= target, measured at sample counts growing by ~10%.

    `ms` is the cumulative device time of all samples up to that point, the time a
    progressive renderer needs to reach the target."""
    import torch
    H, W = scene.host.height, scene.host.width
    acc = torch.zeros((H, W, 3), dtype=torch.float64, device=f"cuda:{scene.ctx.device}")
    curve = []
    have, ms = 0, 0.0
    hit = None
    dropped = [0]
    for spp in checkpoints(first, max_spp):
        ms += _accumulate(scene, acc, seed, have, spp - have, chunk, dropped)
        have = spp
        e = relmse((acc / float(spp)).cpu().numpy(), ref)
        curve.append({"spp": spp, "relmse": e, "ms": ms})
        if e <= target:
            hit = curve[-1]
            break
    return {"target": target, "reached": hit is not None, "spp": hit["spp"] if hit else None,
            "ms": hit["ms"] if hit else None, "dropped_paths": dropped[0], "curve": curve}


def time_to_relmse_cached(scene, cache, ref: np.ndarray, target: float = 1e-3, seed: int = 0,
                          max_spp: int = 1 << 16, frame_spp: int = 4, bounce: int = 2, train_stride: int = 16,
                          train_steps: int = 4, train_batch: int = 1 << 16, train_suffix: int = 0) -> dict:
    """Progressive rendering with the radiance cache trained online: frames of `frame_spp`
    samples, each rendered with the cache as it stands and then used for `train_steps`
    optimiser steps on the frame's training samples. The running FP64 mean of the frames is
    compared with the reference at the same checkpoints as the plain render; `ms` is the
    cumulative device time of the frames (path kernel, network inference, training)."""
    acc = np.zeros_like(ref, dtype=np.float64)
    curve = []
    have, ms = 0, 0.0
    checks = checkpoints(frame_spp, max_spp)
    ci = 0
    parts = {"path_ms": 0.0, "infer_ms": 0.0, "train_ms": 0.0, "queries": 0, "train_samples": 0, "paths": 0}
    hit = None
    while have < max_spp and ci < len(checks):
        img, st, cst = scene.render_cached(cache, bounce=bounce, train_stride=train_stride, train_steps=train_steps,
                                           train_batch=train_batch, seed=seed, spp=frame_spp, sample_offset=have,
                                           train_suffix=train_suffix)
        ms += st["total_ms"]
        for k in ("path_ms", "infer_ms", "train_ms", "queries", "train_samples"):
            parts[k] += cst[k]
        parts["paths"] += st["paths"]
        finite = np.isfinite(img)
        acc += np.where(finite, img, 0.0) * frame_spp
        have += frame_spp
        if have >= checks[ci]:
            ci += 1
            e = relmse(acc / have, ref)
            curve.append({"spp": have, "relmse": e, "ms": ms, "loss": cst["loss"]})
            if e <= target:
                hit = curve[-1]
                break
    return {"target": target, "reached": hit is not None, "spp": hit["spp"] if hit else None,
            "ms": hit["ms"] if hit else None, "frame_spp": frame_spp, "bounce": bounce, "train_suffix": train_suffix,
            "train_stride": train_stride, "train_steps": train_steps, "train_batch": train_batch, "totals": parts,
            "curve": curve}


def main(argv=None):
    import narvalengine_gb300 as ne
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--scene", default="medium_c2")
    ap.add_argument("--ref-spp", type=int, default=65536)
    ap.add_argument("--chunk", type=int, default=256)
    ap.add_argument("--target", type=float, default=1e-3)
    ap.add_argument("--resolution", type=int, nargs=2, default=None, help="override width height")
    ap.add_argument("--save", default=None, help="write the reference image (.npy)")
    ap.add_argument("--cache", action="store_true", help="also measure the radiance-cache form")
    ap.add_argument("--max-spp", type=int, default=1 << 16)
    ap.add_argument("--frame-spp", type=int, default=16)
    ap.add_argument("--bounce", type=int, nargs="+", default=[2], help="cache termination bounce(s) to measure")
    ap.add_argument("--train-steps", type=int, default=4)
    ap.add_argument("--train-stride", type=int, default=16)
    ap.add_argument("--train-suffix", type=int, nargs="+", default=[0],
                    help="bounces a training path runs past its recorded vertex before it ends in the cache too "
                         "(0: to its end); each value is measured")
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
    tuning, _ = scene.autotune(repeats=1, seed=3, spp=args.chunk)
    t0 = time.time()
    info = {}
    ref, ref_ms = reference_image(scene, args.ref_spp, chunk=args.chunk, info=info)
    if args.save:
        np.save(args.save, ref)
    res = time_to_relmse(scene, ref, args.target, chunk=args.chunk, max_spp=args.max_spp)
    if args.cache:
        res["cache"] = []
        for bounce in args.bounce:
            for suffix in args.train_suffix:
                cache = ne.RadianceCache(ctx, seed=1)
                r = time_to_relmse_cached(scene, cache, ref, args.target, max_spp=args.max_spp,
                                          frame_spp=args.frame_spp, bounce=bounce, train_steps=args.train_steps,
                                          train_stride=args.train_stride, train_suffix=suffix)
                cache.close()
                if res["reached"] and r["reached"]:
                    r["time_ratio_vs_plain"] = r["ms"] / res["ms"]
                res["cache"].append(r)
    out = {"scene": os.path.basename(path), "resolution": [host.width, host.height], "ref_spp": args.ref_spp,
           "ref_paths": host.width * host.height * args.ref_spp, "ref_device_ms": ref_ms,
           "ref_wall_s": time.time() - t0, "ref_dropped_paths": info["dropped_paths"], "relmse_eps": EPS,
           "tuning": tuning, **res}
    print(json.dumps(out))
    scene.close()
    ctx.close()


if __name__ == "__main__":
    main()
