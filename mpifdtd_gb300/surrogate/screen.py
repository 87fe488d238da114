"""Training, evaluation and audited screening of the far-field surrogate.

screen() is the sweep path with the network: predict every structure, audit
a fraction of them with the batched FDTD engine, and fall back to FDTD for a
whole screening batch when an audited structure's relative far-field error is
above the tolerance.  The error of a structure is the relative L2 norm of its
31 x 360 far-field intensity against FDTD.
"""
from __future__ import annotations

import math
import time

import numpy as np

from .data import Generator, make_maps
from .model import FNO


def rel_err(pred, ref):
    """Per-structure relative L2 error of [N, 31, 360] intensities."""
    p = np.asarray(pred, np.float64).reshape(len(pred), -1)
    r = np.asarray(ref, np.float64).reshape(len(ref), -1)
    return np.linalg.norm(p - r, axis=1) / np.linalg.norm(r, axis=1)


def generate(n, seed, gen: Generator):
    """n maps and their FDTD far fields; returns (maps, intensity, seconds)."""
    maps = make_maps(n, seed)
    t = gen.seconds
    inten = gen.far_field(maps)
    return maps, inten, gen.seconds - t


def mirror(maps, inten):
    """The mirror image of each structure in y and its far field: with the
    plane wave along x, y -> -y maps the far-field angle phi to -phi."""
    ang = (360 - np.arange(360)) % 360
    return maps[:, :, ::-1].copy(), np.asarray(inten)[:, :, ang].copy()


def shift_ranges(maps, margin=6):
    """Per map the integer shifts (dx_lo, dx_hi, dy_lo, dy_hi) that keep its
    structure at least `margin` cells inside the map (the NTFF path runs 5
    cells inside the map's edge); a structure already closer stays put on
    that side."""
    g = maps.shape[1]
    out = np.zeros((len(maps), 4), np.int64)
    for q, m in enumerate(maps):
        xs = np.nonzero(m.any(axis=1))[0]
        ys = np.nonzero(m.any(axis=0))[0]
        if len(xs) == 0:
            continue
        for a, (lo, hi) in enumerate(((xs[0], xs[-1]), (ys[0], ys[-1]))):
            out[q, 2 * a] = min(0, margin - lo)
            out[q, 2 * a + 1] = max(0, (g - 1 - margin) - hi)
    return out


def shifted(dev_maps, idx, ranges, rng):
    """dev_maps[idx] each translated by a random in-range (dx, dy): the
    far-field intensity of a translated structure is the same (the plane wave
    and the far field only change phase), measured on FDTD data to 0.5 %
    median (shifts up to 100 cells)."""
    import torch
    r = ranges[idx]
    dx = rng.integers(r[:, 0], r[:, 1] + 1)
    dy = rng.integers(r[:, 2], r[:, 3] + 1)
    g = dev_maps.shape[1]
    ar = np.arange(g)
    xi = torch.tensor((ar[None, :] - dx[:, None]) % g, device="cuda")
    yi = torch.tensor((ar[None, :] - dy[:, None]) % g, device="cuda")
    b = torch.tensor(idx, device="cuda")
    return dev_maps[b[:, None, None], xi[:, :, None], yi[:, None, :]].contiguous()


def train(net: FNO, maps, inten, steps=400, batch=128, lr=6e-4, seed=0, log=None, target="rel", augment=True,
          wd=0.0, shift=True):
    """Adam (cosine-decayed learning rate) on minibatches of normalised far
    fields, the training set doubled by its mirror images; with `shift` every
    minibatch structure is also translated at random within the map (same
    far-field intensity).  target "rel" (default) weights each structure's
    squared error by 1 / |its intensity|^2, floored so that no weight exceeds
    20x the mean (a weakly scattering structure's weight otherwise spikes the
    gradients; 6-layer runs at lr 1e-3 diverged without it): the loss is the
    evaluation's per-structure relative L2 error, squared.  Returns seconds."""
    import torch
    if augment:
        mm, mi = mirror(maps, inten)
        maps = np.concatenate([maps, mm])
        inten = np.concatenate([inten, mi])
    target_mode = target
    dev_maps = torch.tensor(maps, device="cuda")
    target = torch.tensor(inten, device="cuda")
    net.set_normalisation(target, target=target_mode)
    y_all = net.encode(target)
    w_all = None
    if target_mode == "rel":
        sq = (y_all.double() ** 2).mean(1)
        w_all = (sq.mean() / (sq + 0.05 * sq.mean())).float().contiguous()
    x_all = None if shift else net.pool(dev_maps)
    ranges = shift_ranges(maps) if shift else None
    n = len(maps)
    rng = np.random.default_rng(seed)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for it in range(steps):
        pick = rng.choice(n, batch, replace=n < batch)
        idx = torch.tensor(pick, device="cuda")
        frac = it / max(1, steps - 1)
        step_lr = lr * 0.5 * (1 + math.cos(math.pi * frac))  # cosine decay
        x = net.pool(shifted(dev_maps, pick, ranges, rng)) if shift else x_all[:, idx].contiguous()
        loss, g = net.loss_and_grads(x, y_all[idx].contiguous(), None if w_all is None else w_all[idx].contiguous())
        net.adam_step(g, lr=step_lr, wd=wd)
        if log is not None and (it % 100 == 0 or it == steps - 1):
            log(it, float(loss.mean()))
    torch.cuda.synchronize()
    return time.perf_counter() - t0


def predict(net: FNO, maps, views=1, seed=11):
    """Far-field intensity [N, 31, 360] of host maps.  views > 1 averages the
    network over symmetric views of each structure, whose far-field
    intensities are the same up to the known angle map: its mirror image
    (y -> -y, phi -> -phi) and views - 2 random translations."""
    import torch
    dev = torch.tensor(maps, device="cuda")
    pred = net.predict(dev)
    if views <= 1:
        return pred.cpu().numpy()
    ang = torch.tensor((360 - np.arange(360)) % 360, device="cuda")
    acc = pred + net.predict(torch.flip(dev, dims=[2]).contiguous())[:, :, ang]
    if views > 2:
        ranges = shift_ranges(np.asarray(maps))
        rng = np.random.default_rng(seed)
        idx = np.arange(len(maps))
        for _ in range(views - 2):
            acc += net.predict(shifted(dev, idx, ranges, rng))
    return (acc / views).cpu().numpy()


def evaluate(net: FNO, maps, inten, train_inten=None, views=1):
    """Errors of the network and of the network-free baseline (the mean
    far field of the training set, the best constant prediction)."""
    pred = predict(net, maps, views)
    err = rel_err(pred, inten)
    out = {"median": float(np.median(err)), "p90": float(np.percentile(err, 90)),
           "within_2pct": float(np.mean(err <= 0.02)), "n": int(len(err))}
    if train_inten is not None:
        base = np.broadcast_to(np.asarray(train_inten).mean(0), inten.shape)
        be = rel_err(base, inten)
        out["baseline_mean_far_field"] = {"median": float(np.median(be)), "p90": float(np.percentile(be, 90)),
                                          "within_2pct": float(np.mean(be <= 0.02))}
    return out


def inference_rate(net: FNO, n=16384, batch=4096, seed=99):
    """Structures per second of the network alone (maps already on the GPU,
    one view per structure)."""
    import torch
    maps = torch.tensor(make_maps(min(n, 512), seed), device="cuda")
    reps = (n + len(maps) - 1) // len(maps)
    maps = maps.repeat(reps, 1, 1)[:n].contiguous()
    net.predict(maps[:batch], batch=batch)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    net.predict(maps, batch=batch)
    torch.cuda.synchronize()
    return n / (time.perf_counter() - t0)


def screen(net: FNO, maps, gen: Generator, audit_frac=0.01, tol=0.02, batch=4096, seed=7, audit_gen=None,
           views=1):
    """Audited surrogate screening.  Per screening batch: predict all (views:
    see predict), run FDTD on ceil(audit_frac * batch) random structures
    (audit_gen: a generator sized for the audit), and if any of them is off
    by more than tol, replace the batch by FDTD (gen).  Returns (intensity,
    stats)."""
    rng = np.random.default_rng(seed)
    audit_gen = audit_gen or gen
    out = np.zeros((len(maps), 31, 360), np.float32)
    stats = {"batches": 0, "fallback_batches": 0, "audited": 0, "audit_errors": [], "seconds": 0.0}
    t0 = time.perf_counter()
    for s in range(0, len(maps), batch):
        part = maps[s:s + batch]
        pred = predict(net, part, views)
        k = max(1, int(math.ceil(audit_frac * len(part))))
        pick = rng.choice(len(part), k, replace=False)
        ref = audit_gen.far_field(part[pick])
        e = rel_err(pred[pick], ref)
        stats["batches"] += 1
        stats["audited"] += k
        stats["audit_errors"] += [float(v) for v in e]
        if (e > tol).any():
            stats["fallback_batches"] += 1
            pred = gen.far_field(part)
        else:
            pred[pick] = ref
        out[s:s + len(part)] = pred
    stats["seconds"] = time.perf_counter() - t0
    stats["structures_per_s"] = len(maps) / stats["seconds"]
    return out, stats
