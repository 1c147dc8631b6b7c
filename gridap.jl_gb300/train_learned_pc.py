"""Trains the learned block preconditioner and writes data/learned_pc_q1_lognormal.npy.

Residual / error pairs come from FP64 CG solves of 200 independent lognormal kappa draws
(seeds 5000..5199, 64^3 cells, correlation length 8 cells, contrast 1e4): the solution x*
to 1e-12, then CG iterates x_k from x0 = x* + white noise (k = 0, 1, 2, 4), inputs from
r_k = b - A x_k and targets e_k = x* - x_k. The network is fitted with the library's FP32
training kernels. Needs a GPU:

    python gridap.jl_gb300/train_learned_pc.py [--n 64] [--draws 200] [--out PATH]
"""
import argparse
import json
import pathlib
import sys
import time

ROOT = pathlib.Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def main():
    import numpy as np

    import __graft_entry__ as ge
    ge.load_package()
    from gridap_gb300 import learned

    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--draws", type=int, default=200)
    ap.add_argument("--epochs", type=int, default=40)
    ap.add_argument("--out", default=str(learned.WEIGHTS_FILE))
    a = ap.parse_args()
    t0 = time.time()
    params, loss = learned.train(n=a.n, draws=a.draws, epochs=a.epochs)
    out = pathlib.Path(a.out)
    out.parent.mkdir(parents=True, exist_ok=True)
    np.save(out, params.astype(np.float32))
    print(json.dumps({"weights": str(out), "loss": loss, "seconds": time.time() - t0,
                      "n": a.n, "draws": a.draws, "epochs": a.epochs}))


if __name__ == "__main__":
    main()
