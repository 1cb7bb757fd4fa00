"""Learned rotation proposal: the network's CPU restatement, the GPU kernels'
gradients against it, training, and pruning.

Tolerances: the FP64 restatement's own gradient agrees with central finite
differences to 1e-5 relative (no BF16 rounding); the GPU's forward values and
per-tensor gradients agree with the restatement (which rounds to BF16 where
the GPU stores BF16) to 2e-3 relative (the fc2 weights' gradient 6e-3), the
gap left by FP32 accumulation order and the occasional BF16 rounding flip it
causes.
"""
import numpy as np
import pytest

from oracle import proposal_oracle as PO

TENSORS = [name for name, _ in PO.SHAPES]


def _tensor_slices():
    out, o = {}, 0
    for name, shape in PO.SHAPES:
        n = int(np.prod(shape))
        out[name] = slice(o, o + n)
        o += n
    return out


def _rand_rot(rng, n):
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    R = np.empty((n, 3, 3))
    R[:, 0] = np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1)
    R[:, 1] = np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1)
    R[:, 2] = np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1)
    return R


def _toy_samples(seed, n_pairs=2, per_pair=3, n_atoms=80):
    from proddl2_gb300 import synth
    rng = np.random.Generator(np.random.PCG64(seed))
    pairs, samples, targets, ids, rots = [], [], [], [], []
    for k in range(n_pairs):
        lig = synth.molecule(n_atoms, seed * 10 + k).xyz
        lig = lig - synth.diameter_centre(lig)
        rec = synth.molecule(300, seed * 10 + 5 + k)
        desc = PO.descriptor(rec.xyz, rec.element)
        pairs.append((lig, rec, desc))
        for R in _rand_rot(rng, per_pair):
            samples.append((lig, PO.half_width(lig), R, desc))
            targets.append(float(rng.normal()))
            ids.append(k)
            rots.append(R)
    return pairs, samples, np.array(targets), np.array(ids), np.array(rots)


def _with_random_biases(params, seed):
    # zero biases put empty regions exactly on the ReLU kink, where finite
    # differences see a one-sided slope
    rng = np.random.Generator(np.random.PCG64(seed))
    p = params.copy()
    sl = _tensor_slices()
    for name in ("b1", "b2", "b3", "fb1"):
        p[sl[name]] = rng.uniform(-0.05, 0.05, size=sl[name].stop - sl[name].start)
    return p


def test_oracle_gradient_matches_finite_differences():
    params = _with_random_biases(PO.init_params(3), 4)
    _, samples, targets, _, _ = _toy_samples(1, n_pairs=1, per_pair=2, n_atoms=40)
    loss, g, _ = PO.forward_backward(params, samples, targets, bf=False)
    rng = np.random.Generator(np.random.PCG64(9))
    sl = _tensor_slices()
    ok = total = 0
    for name in TENSORS:
        idx = rng.choice(np.arange(sl[name].start, sl[name].stop), size=min(6, sl[name].stop - sl[name].start),
                         replace=False)
        for i in idx:
            h = 1e-6 * max(1.0, abs(params[i]))
            p1, p2 = params.copy(), params.copy()
            p1[i] += h
            p2[i] -= h
            fd = (PO.forward_backward(p1, samples, targets, bf=False)[0]
                  - PO.forward_backward(p2, samples, targets, bf=False)[0]) / (2 * h)
            total += 1
            if abs(fd - g[i]) <= 1e-5 * max(1e-3, abs(fd), abs(g[i])):
                ok += 1
    # a perturbation that crosses a ReLU kink may miss; nothing else may
    assert ok >= total - 2, (ok, total)


def test_descriptor_matches_oracle(built_lib):
    from proddl2_gb300 import synth
    from proddl2_gb300.proposal import receptor_descriptor
    rec = synth.molecule(2500, 77)
    d = receptor_descriptor(rec.xyz, rec.element)
    ref = PO.descriptor(rec.xyz, rec.element)
    assert np.allclose(d, ref, rtol=0, atol=1e-7)
    assert abs(d.sum() - 1.0) < 1e-5


def test_oriented_descriptor_matches_oracle(built_lib):
    from proddl2_gb300 import synth
    from proddl2_gb300.proposal import receptor_descriptor_oriented
    rec = synth.molecule(2500, 78)
    d = receptor_descriptor_oriented(rec.xyz)
    ref = PO.descriptor_oriented(rec.xyz)
    assert np.allclose(d, ref, rtol=0, atol=1e-7)
    assert abs(d[:64].sum() - 1.0) < 1e-5 and 0 < d[64:].sum() < 1
    # the frame matters: a rotated receptor gives a different input
    R = np.array([[0.0, -1.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, 1.0]])
    assert not np.allclose(receptor_descriptor_oriented(rec.xyz @ R.T), d)
    assert np.all(receptor_descriptor_oriented(np.zeros((0, 3))) == 0)


def test_pruning_helpers():
    from proddl2_gb300.proposal import keep_best, recall, standardize
    z = standardize(np.array([-5.0, -1.0, np.inf, -3.0]))
    assert z[2] == 3.0 and np.argmin(z) == 0
    assert list(keep_best(np.array([0.3, -1.0, 2.0, -0.5, 0.0]), 0.4)) == [1, 3]
    a = [(-3.0, 1, (0, 0, 0)), (-2.0, 4, (1, 0, 0))]
    b = [(-3.0, 1, (0, 0, 0)), (-1.0, 7, (1, 0, 0))]
    assert recall(a, b) == 0.5


@pytest.mark.gpu
def test_gpu_forward_and_gradients_match_oracle():
    from proddl2_gb300.proposal import Proposal
    pairs, samples, targets, ids, rots = _toy_samples(5, n_pairs=2, per_pair=3)
    with Proposal(seed=11) as p:
        pid = [p.add_pair(lig, desc=desc) for lig, _, desc in pairs]
        params = p.params.astype(np.float64)
        g, loss = p.gradients(np.array(pid)[ids], rots, targets)
        pred = np.concatenate([p.predict(pid[k], rots[ids == k]) for k in range(len(pairs))])
    ref_loss, ref_g, ref_pred = PO.forward_backward(params, samples, targets, bf=True)
    order = np.concatenate([np.nonzero(ids == k)[0] for k in range(len(pairs))])
    assert np.allclose(pred, ref_pred[order], rtol=2e-3, atol=2e-3 * np.abs(ref_pred).max())
    assert abs(loss - ref_loss) <= 2e-3 * max(1.0, ref_loss)
    sl = _tensor_slices()
    rel = {}
    for name in TENSORS:
        a, b = g[sl[name]].astype(np.float64), ref_g[sl[name]]
        nb = np.linalg.norm(b)
        assert nb > 0, name
        rel[name] = float(np.linalg.norm(a - b) / nb)
    print("relative gradient error per tensor:", {k: "%.1e" % v for k, v in rel.items()})
    for name, r in rel.items():
        # f2's gradient sums dy * h1 over only 6 samples with strong
        # cancellation, and h1 is rounded to BF16: one rounding flip of an h1
        # element (a 2^-8 step, caused by FP32 accumulation order) moves an
        # entry by ~2e-4 absolute, so its bar is wider
        assert r <= (6e-3 if name == "f2" else 2e-3), (name, r)


@pytest.mark.gpu
def test_training_lowers_the_loss_and_params_round_trip():
    from proddl2_gb300.proposal import Proposal
    pairs, _, _, _, _ = _toy_samples(6, n_pairs=2, per_pair=1)
    rng = np.random.Generator(np.random.PCG64(2))
    with Proposal(seed=1) as p:
        pid = [p.add_pair(lig, desc=desc) for lig, _, desc in pairs]
        for k, (lig, _, _) in enumerate(pairs):
            R = _rand_rot(rng, 512)
            # a learnable target: the rotated ligand's x extent
            t = np.array([(lig @ r.T)[:, 0].max() for r in R]) / 10.0
            p.add_samples(pid[k], R, t)
        first = p.train(20, batch=128, lr=1e-3, seed=3)
        for _ in range(10):
            last = p.train(40, batch=128, lr=1e-3, seed=3)
        assert last < 0.5 * first, (first, last)
        w = p.params
        p.params = w
        assert np.array_equal(p.params, w)


@pytest.mark.gpu
def test_pruning_gain_over_random_on_a_learnable_score():
    """What the trained network gains over pruning without it (a random
    subset of the same size), on a score that a rotation-level predictor can
    learn: the rotated ligand's extent along x.  Held-out rotations only."""
    from proddl2_gb300 import synth
    from proddl2_gb300.proposal import Proposal, keep_best
    lig = synth.molecule(450, 4242).xyz
    lig = lig - synth.diameter_centre(lig)
    rec = synth.molecule(2500, 4243)
    rot = synth.quaternion_rotations(3000, seed=17)
    score = -np.array([(lig @ r.T)[:, 0].max() for r in rot])   # lower is better
    z = (score - score.mean()) / score.std()
    train, test = np.arange(2000), np.arange(2000, 3000)
    with Proposal(seed=2) as p:
        pid = p.add_pair(lig, rec.xyz, rec.element)
        p.add_samples(pid, rot[train], z[train])
        for _ in range(6):
            p.train(250, batch=256, lr=1e-3, seed=5)
        pred = p.predict(pid, rot[test])
    best = set(test[np.argsort(score[test])[:50]])          # the 50 best held-out rotations
    kept = set(test[keep_best(pred, 0.2)])
    learned = len(best & kept) / 50
    rng = np.random.Generator(np.random.PCG64(0))
    rand = np.mean([len(best & set(rng.choice(test, 200, replace=False))) / 50 for _ in range(20)])
    print("top-50 recall at 20%% kept: learned %.2f, random %.2f" % (learned, rand))
    assert learned >= 0.6 and learned >= 2.5 * rand
