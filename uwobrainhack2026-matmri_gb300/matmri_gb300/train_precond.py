"""Trains the learned CG-SENSE preconditioner on pairs generated by plain CG.

    python -m matmri_gb300.train_precond [--train 4000] [--val 500] [--steps 3000] [--out PATH]

Workload: 256 x 256 image, 32 coils with randomised ring-of-Gaussians maps,
4 x 4096 variable-density spiral at R = 4 (kwidth 4, os 2), random-ellipse
phantoms with a smooth complex phase, complex Gaussian noise at SNR 30.

System: the Tikhonov-regularised normal equations cgne solves with gam = lam
and R = 1 (cgne.m:171-179), (A'A + lam) x = A'y, lam = LAM_REL * lambda_max(A'A).
Without regularisation the k-space corners outside the spiral disc are in
the null space of A'A, and the noisy least-squares solution is never reached.

1. Pairs: for every training seed, plain CG from x0 = 0 for NIT_REF
   iterations gives x*; (r_k, x* - x_k) at k in KEEP are the pairs, the map a
   preconditioner should apply (e = (A'A + lam)^-1 r).
2. Training: Adam on random 64 x 64 crops of the pairs (crops may reach past
   the image, zero-filled, so image-border pixels are trained too); the loss
   drops the 6 pixels next to each crop edge (the receptive-field radius) and
   is scale invariant (1 - cosine^2).  The network is linear (identity
   activations): a fixed operator keeps flexible CG as strong as PCG.
3. Validation on held-out seeds: iterations to NRMSE <= 1e-3 against x* for
   plain CG and for the learned PCG, both from x0 = 0.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import time

import numpy as np

N, NC, N_INT, N_SAMP, ACCEL, SNR = 256, 32, 4, 4096, 4.0, 30.0
LAM_REL = 1e-3
NIT_REF = 160
KEEP = (0, 3, 8, 16, 30, 50, 80, 110)
TRAIN_SEED0, VAL_SEED0 = 100_000, 200_000
WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "precond_256x32_r4.npz")


def make_operator_base(device):
    """The shared nufftOp of the workload (the trajectory does not depend on the seed)."""
    import matmri_gb300 as mm
    from matmri_gb300 import synth
    kloc = synth.spiral(N, N_INT, N_SAMP, ACCEL)
    return mm.nufftOp([N, N], kloc, None, 1, 2.0, 4)


def make_case(S, seed, device):
    """(A, y, img) for one seed: phantom, randomised maps and SNR-30 noise, all on the device."""
    import torch
    import matmri_gb300 as mm
    from matmri_gb300 import synth
    img = synth.ellipse_phantom_torch(N, 10, seed, complex_phase=True, device=device)
    maps = synth.coil_maps_torch(N, NC, seed + 1, randomize=True, device=device)
    R = mm.rcvrOp(maps.cpu().numpy(), 0)
    A = mm.mrSampOp(S, R)
    y = A(img, "notransp")
    g = torch.Generator(device=device)
    g.manual_seed(int(seed) * 7 + 1)
    sig = float(torch.sqrt((y.abs() ** 2).mean())) / SNR
    nz = torch.complex(torch.randn(y.shape, generator=g, device=device),
                       torch.randn(y.shape, generator=g, device=device)) * (sig / math.sqrt(2))
    return A, y + nz, img


def lambda_max(A, device, iters=40, seed=0):
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    v = torch.complex(torch.randn((N, N), generator=g, device=device), torch.randn((N, N), generator=g, device=device))
    v = v.T.contiguous().T
    lm = 0.0
    for _ in range(iters):
        w = A.normal(v)
        lm = float(torch.linalg.norm(w)) / float(torch.linalg.norm(v))
        v = w / torch.linalg.norm(w)
    return lm


def reference_solution(A, b, lam, nit=NIT_REF, keep=()):
    from matmri_gb300.learned import cg_iterates
    return cg_iterates(A.normal, b, lam, nit, set(keep))


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=4000)
    ap.add_argument("--val", type=int, default=500)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--report", default=None)
    args = ap.parse_args(argv)
    import torch
    import matmri_gb300 as mm
    from matmri_gb300.learned import PrecondNet, iterations_to, lpcg, train
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    S = make_operator_base(dev)
    A0, _, _ = make_case(S, TRAIN_SEED0, dev)
    lmax = lambda_max(A0, dev)
    lam = LAM_REL * lmax
    del A0
    print(f"lambda_max {lmax:.4f}, lam {lam:.5f}", flush=True)
    report = {"lambda_max": lmax, "lam": lam, "lam_rel": LAM_REL, "nit_ref": NIT_REF, "keep": list(KEEP),
              "train_seeds": args.train, "val_seeds": args.val}

    # 1. pairs from plain CG
    t0 = time.time()
    npair = args.train * len(KEEP)
    Rp = torch.empty((npair, N, N), dtype=torch.complex64, device=dev)
    Ep = torch.empty((npair, N, N), dtype=torch.complex64, device=dev)
    j = 0
    for i in range(args.train):
        A, y, _ = make_case(S, TRAIN_SEED0 + i, dev)
        b = A(y, "transp")
        xs, kept = reference_solution(A, b, lam, keep=KEEP)
        for k in KEEP:
            rk, xk = kept[k]
            Rp[j] = rk
            Ep[j] = xs - xk
            j += 1
        del A
        if i % 500 == 0:
            print(f"pairs: seed {i}/{args.train} ({time.time() - t0:.1f} s)", flush=True)
    torch.cuda.synchronize()
    report["pair_gen_s"] = time.time() - t0

    # 2. training
    net = PrecondNet(seed=1)
    t0 = time.time()
    losses = train(net, Rp, Ep, steps=args.steps, batch=args.batch, lr=args.lr, seed=2, log_every=250)
    torch.cuda.synchronize()
    report["train_s"] = time.time() - t0
    report["loss_first"] = float(np.mean(losses[:20]))
    report["loss_last"] = float(np.mean(losses[-50:]))
    del Rp, Ep
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    net.save(args.out, lam_rel=LAM_REL, lam=lam, lambda_max=lmax, train_seeds=args.train, steps=args.steps)

    # 3. validation
    t0 = time.time()
    its_plain, its_learn, fell = [], [], 0
    ms = {"plain": [], "learned": []}
    for i in range(args.val):
        A, y, _ = make_case(S, VAL_SEED0 + i, dev)
        b = A(y, "transp")
        xs, _ = reference_solution(A, b, lam)
        gn = float(torch.linalg.norm(xs))
        res = {}
        for name, nn in (("plain", None), ("learned", net)):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            _, _, err, info = lpcg(A, y, nn, NitMax=80, lam=lam, gtruth=xs)
            e1.record()
            torch.cuda.synchronize()
            ms[name].append(e0.elapsed_time(e1))
            res[name] = (iterations_to(err, gn), info)
        its_plain.append(res["plain"][0])
        its_learn.append(res["learned"][0])
        fell += res["learned"][1]["fell_back_at"] >= 0
        del A
    report["val_ms_per_80it_plain"] = float(np.median(ms["plain"]))
    report["val_ms_per_80it_learned"] = float(np.median(ms["learned"]))
    report["val_s"] = time.time() - t0
    ok = [(p, l) for p, l in zip(its_plain, its_learn) if p is not None and l is not None]
    report["val_reached_plain"] = sum(p is not None for p in its_plain)
    report["val_reached_learned"] = sum(l is not None for l in its_learn)
    report["val_fell_back"] = fell
    if ok:
        p, l = np.array(ok, dtype=float).T
        report["val_its_plain_median"] = float(np.median(p))
        report["val_its_learned_median"] = float(np.median(l))
        report["val_its_ratio_mean"] = float(np.mean(l / p))
    print(json.dumps(report), flush=True)
    if args.report:
        with open(args.report, "w") as f:
            json.dump(report, f, indent=1)


if __name__ == "__main__":
    main()
