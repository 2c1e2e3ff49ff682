"""Throughput of the radiance-cache network kernels on the tensor cores.

    python -m narvalengine_gb300.cache_bench [--queries 16777216] [--batch 65536] [--steps 20]

Inference: `queries` random queries (object-space position, unit direction) resident on the
device, encoded and run through the five layers by k_mlp_forward. Training: Adam steps on
`batch` samples (forward with stored activations, backward with weight-gradient products
accumulated in tensor memory, reduction + Adam, BF16 repacking). Times are CUDA events on the
library's stream after warm-up. Algorithmic FLOPs count the products only, without the padding
rows and columns the kernels carry: forward 2 x (96*64 + 3*64*64 + 64*3) per query; a
training sample adds the error products 2 x (3*64 + 3*64*64) and the weight-gradient products
2 x (96*64 + 3*64*64 + 64*3).
"""
from __future__ import annotations

import argparse
import json

import numpy as np

FWD_FLOPS = 2 * (96 * 64 + 3 * 64 * 64 + 64 * 3)
BWD_FLOPS = 2 * (3 * 64 + 3 * 64 * 64) + FWD_FLOPS
TRAIN_FLOPS = FWD_FLOPS + BWD_FLOPS


def main(argv=None):
    import torch
    import narvalengine_gb300 as ne
    from narvalengine_gb300 import _abi
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--queries", type=int, default=1 << 24)
    ap.add_argument("--batch", type=int, default=1 << 16)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    args = ap.parse_args(argv)
    ctx = ne.Context(0)
    cache = ne.RadianceCache(ctx, seed=1)
    lib = ne.library()
    g = torch.Generator(device="cuda:0").manual_seed(7)
    n = args.queries
    pos = torch.rand((n, 3), device="cuda:0", generator=g) - 0.5
    d = torch.randn((n, 3), device="cuda:0", generator=g)
    d = d / d.norm(dim=1, keepdim=True)
    out = torch.empty((n, 3), device="cuda:0")
    tgt = torch.rand((args.batch, 3), device="cuda:0", generator=g) + 0.2
    dev = _abi.NE_CACHE_DEVICE_PTRS

    def infer():
        ctx.check(lib.ne_cache_infer(cache._h, pos.data_ptr(), d.data_ptr(), None, n, out.data_ptr(), dev))

    def train():
        ctx.check(lib.ne_cache_train(cache._h, pos.data_ptr(), d.data_ptr(), None, tgt.data_ptr(), args.batch, 1,
                                     None, None, dev))

    res = {}
    for name, fn, units, flops in (("inference", infer, n, FWD_FLOPS), ("training", train, args.batch, TRAIN_FLOPS)):
        for _ in range(args.warmup):
            fn()
        ctx.synchronize()
        ctx.record(0)
        for _ in range(args.steps):
            fn()
        ctx.record(1)
        ms = ctx.elapsed_ms(0, 1) / args.steps
        res[name] = {"units_per_call": units, "ms_per_call": ms, "units_per_s": units / (ms / 1e3),
                     "algorithmic_tflops": units * flops / (ms / 1e3) / 1e12}
    print(json.dumps(res))
    cache.close()
    ctx.close()


if __name__ == "__main__":
    main()
