"""A few Lanczos steps of a named workload, for profilers.

    python -m tdscha_gb300.profile_step [--workload m573_n20k] [--precision mixed]
                                        [--warmup 3] [--steps 4] [--stage-a-acc 0|1]

Builds the context of the workload's seeded synthetic ensemble (the shapes of
tdscha_gb300.synthetic.WORKLOADS), runs `warmup` bi-Lanczos steps with full
re-biorthogonalisation, then `steps` more, and prints the kernel launch
counts of one application.  Meant to run under ncu with a kernel filter
(-k) and a launch skip (-s) that passes over the set-up and warm-up launches.
"""
import argparse
import ctypes
import os

import numpy as np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="m573_n20k")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--stage-a-acc", type=int, default=None, choices=[0, 1],
                    help="fix the stage A kernel (1: one accumulator) instead of tuning it")
    args = ap.parse_args()
    if args.stage_a_acc is not None:
        os.environ["TDSCHA_STAGEA_ACC"] = str(args.stage_a_acc)
    import torch
    from . import _native as nat
    from .synthetic import WORKLOADS, make_ensemble, random_R1
    spec = WORKLOADS[args.workload]
    ens = make_ensemble(spec["M"], spec["N"], seed=2024, n_syms=spec["n_syms"],
                        rho_sigma=spec["rho_sigma"])
    M = spec["M"]
    if spec["n_syms"] > 1:
        syms, spaces, bid = ens["symmetries"], ens["degenerate_space"], ens["sym_block_id"]
    else:
        syms = [np.ones((1, 1, 1))] * M
        spaces = [np.array([i], dtype=np.intc) for i in range(M)]
        bid = np.arange(M, dtype=np.intc)
    mixed = args.precision == "mixed"
    ctx = nat.Context(ens["X"], ens["Y"], ens["w"], ens["rho"], ens["T"], syms, spaces, bid,
                      with_mixed=mixed)
    ctx.set_options(False, False, False, False, False, 0.0)
    P = ctx.P
    cap = args.warmup + args.steps + 2
    dev = torch.device("cuda")
    ld = ctx.basis_ld()                  # rows padded to 256 bytes
    ctx.set_basis_ld(ld)
    Qd = torch.empty((cap, ld), dtype=torch.float64, device=dev)
    Pd = torch.empty((cap, ld), dtype=torch.float64, device=dev)
    psi = np.zeros(P)
    psi[:M] = random_R1(M, 11)
    first = torch.from_numpy(psi / np.linalg.norm(psi)).to(dev)
    Qd[0, :P].copy_(first)
    Pd[0, :P].copy_(first)
    hist = np.zeros(4 * cap)
    hist[3] = 1.0
    done, conv = ctypes.c_int(0), ctypes.c_int(0)
    lib = nat.load()
    prec = nat.PREC_MIXED if mixed else nat.PREC_FP64
    st = torch.cuda.current_stream().cuda_stream
    start = 0
    for n in (args.warmup, args.steps):
        nat.check(lib.tdscha_lanczos_run(ctx.handle, Qd.data_ptr(), Pd.data_ptr(), cap, start, n,
                                         0, prec, 1, nat.dp(hist), ctypes.byref(done),
                                         ctypes.byref(conv), st))
        start += n
    torch.cuda.synchronize()
    info = {"workload": args.workload, "precision": args.precision, "layout": ctx.layout()}
    if mixed:
        info["tuning"] = ctx.tuning()
    print(info)
    ctx.close()


if __name__ == "__main__":
    main()
