"""Train the learned rotation proposal on exhaustive scan scores and measure
what pruning with it keeps.

    python -m proddl2_gb300.proposal_train --pairs 512 --heldout 64 --out proposal.npy

Training pairs use the shape-only generator of the 64^3 workload with
receptors of 2000-5000 atoms (log-uniform) and 450-atom ligands, scanned at
128^3 over one shared set of uniform rotations; each rotation's target is its
best score standardised within its pair.  Held-out pairs are scanned
exhaustively (the fallback and the judge) and with pruning (predict, keep the
best fraction, scan those); the report gives the top-k pose recall, the
recall of a random selection of the same size, and the time of both.  One
JSON line goes to stdout.
"""
from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np

from . import synth
from .proposal import (Proposal, best_scores, keep_best, recall, receptor_descriptor,
                       receptor_descriptor_oriented, standardize, top_poses)
from .scan import FFTScan, ScanConfig


def pair_sizes(i, seed):
    rng = np.random.Generator(np.random.PCG64(seed * 1000003 + i))
    n_rec = int(round(math.exp(rng.uniform(math.log(2000), math.log(5000)))))
    return n_rec, 450


def make_pair(i, seed, rotations):
    n_rec, n_lig = pair_sizes(i, seed)
    rec = synth.molecule(n_rec, seed * 7919 + 4 * i + 1)
    lig = synth.molecule(n_lig, seed * 7919 + 4 * i + 2)
    rec.xyz = rec.xyz - synth.box_centre(rec.xyz)
    lig.xyz = lig.xyz - synth.diameter_centre(lig.xyz)
    return synth.Pair(rec, lig, rotations, None)


def scan_config(grid_n, peaks, batch=64):
    return ScanConfig(grid_n=grid_n, grid_step=1.2, term_set="shape", peaks_per_rot=peaks, rot_batch=batch)


def exhaustive(scan, pair, rotations):
    scan.set_receptor(pair.receptor.xyz)
    scan.set_ligand(pair.ligand.xyz)
    return scan.scan(rotations, raise_out_of_grid=False)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--pairs", type=int, default=512)
    ap.add_argument("--heldout", type=int, default=64)
    ap.add_argument("--n-rot", type=int, default=9000)
    ap.add_argument("--grid", type=int, default=128)
    ap.add_argument("--steps", type=int, default=6000)
    ap.add_argument("--batch", type=int, default=256)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--keep", type=float, default=0.2)
    ap.add_argument("--top", type=int, default=100)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--out", default="")
    ap.add_argument("--load", default="", help="skip training: load weights saved by --out")
    ap.add_argument("--descriptor", choices=("radial", "oriented"), default="radial",
                    help="receptor input: radial element histograms or scan-frame occupancy")
    args = ap.parse_args(argv)

    rotations = synth.quaternion_rotations(args.n_rot, seed=args.seed * 31 + 7)
    report = {"pairs": args.pairs, "heldout": args.heldout, "n_rot": args.n_rot, "grid": args.grid,
              "keep": args.keep, "top": args.top, "descriptor": args.descriptor}
    net = Proposal(seed=args.seed)
    with FFTScan(scan_config(args.grid, 4)) as scan:
        if args.load:
            net.load(args.load)
        else:
            t0 = time.perf_counter()
            n_rot_scanned = 0
            for i in range(args.pairs):
                pair = make_pair(i, args.seed, rotations)
                res = exhaustive(scan, pair, rotations)
                n_rot_scanned += len(rotations)
                pid = net.add_pair(pair.ligand.xyz, desc=describe(pair, args.descriptor))
                net.add_samples(pid, rotations, standardize(best_scores(res)))
            report["label_scan_s"] = time.perf_counter() - t0
            t0 = time.perf_counter()
            losses = []
            chunk = max(1, args.steps // 20)
            done = 0
            while done < args.steps:
                k = min(chunk, args.steps - done)
                losses.append(net.train(k, batch=args.batch, lr=args.lr, seed=args.seed))
                done += k
            report["train_s"] = time.perf_counter() - t0
            report["train_loss"] = [round(v, 4) for v in losses]
            net.clear_samples()
            if args.out:
                net.save(args.out)

        # held-out pairs: exhaustive vs pruned
        rng = np.random.Generator(np.random.PCG64(args.seed + 99))
        rec_l, rec_r, t_ex, t_pr, t_pred = [], [], 0.0, 0.0, 0.0
        rho = []
        fracs = (0.2, 0.33, 0.5)
        sweep = {k: {f: [] for f in fracs} for k in ("learned", "random", "neighbour")}
        nearest = nearest_rotation(rotations)
        for j in range(args.heldout):
            pair = make_pair(100000 + j, args.seed, rotations)
            scan.set_receptor(pair.receptor.xyz)
            scan.set_ligand(pair.ligand.xyz)
            scan.scan(rotations[:64], raise_out_of_grid=False)  # warm
            t0 = time.perf_counter()
            full = scan.scan(rotations, raise_out_of_grid=False)
            t_ex += time.perf_counter() - t0
            ref_top = top_poses(full, np.arange(len(rotations)), args.top)
            pid = net.add_pair(pair.ligand.xyz, desc=describe(pair, args.descriptor))
            t0 = time.perf_counter()
            pred = net.predict(pid, rotations)
            keep = keep_best(pred, args.keep)
            t1 = time.perf_counter()
            sub = scan.scan(rotations[keep], raise_out_of_grid=False)
            t2 = time.perf_counter()
            t_pred += t1 - t0
            t_pr += t2 - t0
            rec_l.append(recall(ref_top, top_poses(sub, keep, args.top)))
            rnd = np.sort(rng.choice(len(rotations), size=len(keep), replace=False))
            rec_r.append(recall(ref_top, top_poses(_subset(full, rnd), rnd, args.top)))
            best = best_scores(full)
            fin = np.isfinite(best)
            rho.append(_spearman(pred[fin], best[fin]))
            # the same recall at other kept fractions, read off the exhaustive
            # scan (a rotation's peaks do not depend on the others scanned);
            # "neighbour" ranks each rotation by the true best score of its
            # nearest other rotation: a predictor that knows the score field
            # exactly at the set's spacing
            for f in fracs:
                for kind, score in (("learned", pred), ("random", rng.random(len(rotations))),
                                    ("neighbour", best[nearest])):
                    idx = keep_best(score, f)
                    sweep[kind][f].append(recall(ref_top, top_poses(_subset(full, idx), idx, args.top)))
        report.update({
            "recall_learned_mean": float(np.mean(rec_l)), "recall_learned_min": float(np.min(rec_l)),
            "recall_random_mean": float(np.mean(rec_r)),
            "spearman_pred_vs_best_mean": float(np.mean(rho)),
            "exhaustive_rot_per_s": args.heldout * len(rotations) / t_ex,
            "pruned_rot_per_s_equiv": args.heldout * len(rotations) / t_pr,
            "speedup": t_ex / t_pr,
            "predict_ms_per_pair": 1000.0 * t_pred / args.heldout,
            "recall_by_keep": {kind: {str(f): float(np.mean(v)) for f, v in d.items()} for kind, d in sweep.items()},
        })
    net.close()
    print(json.dumps(report))
    return report


def nearest_rotation(rotations, chunk=1024):
    """Index of each rotation's nearest other rotation (largest trace of
    R_i^T R_j, i.e. smallest rotation angle between them)."""
    r = np.asarray(rotations, dtype=np.float64).reshape(-1, 9)
    out = np.empty(len(r), dtype=np.int64)
    for a in range(0, len(r), chunk):
        t = r[a:a + chunk] @ r.T
        t[np.arange(len(t)), np.arange(a, a + len(t))] = -np.inf
        out[a:a + len(t)] = np.argmax(t, axis=1)
    return out


def describe(pair, kind):
    """The receptor input of the network for one pair."""
    if kind == "oriented":
        return receptor_descriptor_oriented(pair.receptor.xyz)
    return receptor_descriptor(pair.receptor.xyz, pair.receptor.element)


def _subset(result, idx):
    from .scan import ScanResult
    return ScanResult(result.peaks[idx], result.n_peaks[idx], result.status, result.message)


def _spearman(a, b):
    ra = np.argsort(np.argsort(a)).astype(np.float64)
    rb = np.argsort(np.argsort(b)).astype(np.float64)
    ra -= ra.mean()
    rb -= rb.mean()
    d = math.sqrt((ra * ra).sum() * (rb * rb).sum())
    return float((ra * rb).sum() / d) if d > 0 else 0.0


if __name__ == "__main__":
    main()
