"""Train and evaluate the far-field surrogate on data from the batched engine.

    python -m mpifdtd_gb300.surrogate --train 4096 --val 256 --steps 20000

Prints one JSON object: FDTD data-generation rate, training time, held-out
errors (network and network-free baseline), network throughput and the
audited screening of the held-out maps at the given tolerance."""
from __future__ import annotations

import argparse
import json
import sys

import numpy as np


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m mpifdtd_gb300.surrogate")
    ap.add_argument("--train", type=int, default=1024)
    ap.add_argument("--val", type=int, default=256)
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--batch", type=int, default=128)
    ap.add_argument("--lr", type=float, default=6e-4)
    ap.add_argument("--no-shift", action="store_true", help="no random translations of the training maps")
    ap.add_argument("--views", type=int, default=1,
                    help="average the prediction over the structure, its mirror image and views-2 translations")
    ap.add_argument("--seed", type=int, default=20261207)
    ap.add_argument("--tol", type=float, default=0.02)
    ap.add_argument("--mode", choices=["broadband", "cw"], default="broadband",
                    help="FDTD data: one pulse run per map (broadband) or one CW run per wavelength (cw)")
    a = ap.parse_args(argv)
    from .data import Generator
    from .model import FNO
    from . import screen as S
    gen = Generator(group=256 if a.mode == "broadband" else 64, mode=a.mode)
    maps, inten, sec = S.generate(a.train + a.val, a.seed, gen)
    net = FNO(seed=1)
    t_train = S.train(net, maps[:a.train], inten[:a.train], steps=a.steps, batch=a.batch, lr=a.lr,
                      shift=not a.no_shift)
    ev = S.evaluate(net, maps[a.train:], inten[a.train:], inten[:a.train], views=a.views)
    ev1 = ev if a.views <= 1 else S.evaluate(net, maps[a.train:], inten[a.train:])
    rate = S.inference_rate(net)
    k = max(1, int(np.ceil(0.01 * a.val)))
    audit = Generator(group=k, mode=a.mode)
    _, st = S.screen(net, maps[a.train:], gen, audit_frac=0.01, tol=a.tol, batch=a.val, audit_gen=audit,
                     views=a.views)
    out = {"maps": a.train + a.val, "mode": a.mode, "fdtd_structures_per_s": (a.train + a.val) / sec,
           "train": {"maps": a.train, "with_mirror_images": 2 * a.train, "steps": a.steps, "lr": a.lr,
                     "random_translations": not a.no_shift, "seconds": t_train},
           "heldout_rel_l2": ev, "views": a.views, "heldout_rel_l2_one_view": ev1, "network_structures_per_s": rate,
           "network_structures_per_s_with_views": rate / max(1, a.views),
           "screen": {k2: v for k2, v in st.items()}}
    json.dump(out, sys.stdout)
    print()
    audit.close()
    gen.close()


if __name__ == "__main__":
    main()
