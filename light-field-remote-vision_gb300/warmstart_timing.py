"""Times the learned warm start network on one GPU: inference (one image) and a training step (a batch), with
random inputs of the network's shape. Usage:

    python light-field-remote-vision_gb300/warmstart_timing.py [--size 512] [--batch 4] [--reps 10]

Prints one line per measurement (CUDA events on the library's stream, after warm-up).
"""
from __future__ import annotations

import argparse
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parent))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=512)
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--reps", type=int, default=10)
    ap.add_argument("--no-train", action="store_true")
    ap.add_argument("--conv-kernel", type=int, default=None, help="lfrv_set_conv_kernel choice (0, 1, 2)")
    args = ap.parse_args()
    import torch
    import lfrv

    if args.conv_kernel is not None:
        lfrv.set_conv_kernel(args.conv_kernel)
    ctx = lfrv.Context(0)
    net = lfrv.WarmStart(ctx, seed=1)
    H = W = args.size
    B = args.batch
    g = torch.Generator(device="cuda").manual_seed(0)
    x = torch.rand((B, H, W, lfrv.WARMSTART_CHANNELS), device="cuda", generator=g).to(torch.bfloat16)
    u0 = torch.rand((B, 3, H, W), device="cuda", generator=g)
    tg = u0 + 0.01 * torch.randn((B, 3, H, W), device="cuda", generator=g)
    pred = torch.zeros_like(u0)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if not args.no_train:
        for _ in range(2):
            net.train_step_dev(B, H, W, x.data_ptr(), u0.data_ptr(), tg.data_ptr(), 1e-4)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(args.reps):
            net.train_step_dev(B, H, W, x.data_ptr(), u0.data_ptr(), tg.data_ptr(), 1e-4)
        e1.record()
        torch.cuda.synchronize()
        print(f"train step {B} x {H}x{W}: {e0.elapsed_time(e1) / args.reps:.3f} ms", flush=True)
    for _ in range(3):
        net.forward_dev(1, H, W, x[0].data_ptr(), u0[0].data_ptr(), pred[0].data_ptr())
    torch.cuda.synchronize()
    e0.record()
    for _ in range(args.reps):
        net.forward_dev(1, H, W, x[0].data_ptr(), u0[0].data_ptr(), pred[0].data_ptr())
    e1.record()
    torch.cuda.synchronize()
    print(f"forward 1 x {H}x{W}: {e0.elapsed_time(e1) / args.reps:.3f} ms", flush=True)
    net.close()
    ctx.close()


if __name__ == "__main__":
    main()
