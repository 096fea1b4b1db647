"""Voxel-by-voxel agreement of two dose estimates, each given as a per-history
mean with its standard error from independent statistical batches.

The criterion is the one the target states for full dose grids: in the voxels
above 10 % of the maximum dose, each voxel's difference within combined 2
sigma, plus the maximum and mean percent differences. With sigma itself
estimated from B batches, |diff| / sigma follows Student's t rather than the
normal law, so "within 2 sigma" uses the t quantile of the same two-sided
probability as 2 sigma of a normal (95.45 %) at the Welch-Satterthwaite degrees
of freedom of each voxel; that makes the expected fraction 95.45 % for two
unbiased estimates, whatever the batch counts.
"""
import math

import numpy as np

P_2SIGMA = math.erf(2.0 / math.sqrt(2.0))     # 0.9545: two-sided probability of |z| < 2


def batch_estimate(dose, dose2, batches, histories):
    """Per-history mean and its standard error from a run's tallies: dose is
    the sum of the `batches` batch sums t_b, dose2 the sum of t_b^2."""
    dose = np.asarray(dose, dtype=np.float64)
    dose2 = np.asarray(dose2, dtype=np.float64)
    b = float(batches)
    var = np.maximum(dose2 - dose * dose / b, 0.0) / max(b - 1.0, 1.0)   # variance of a batch sum
    return dose / histories, np.sqrt(b * var) / histories


def batches_estimate(batch_doses):
    """Per-history mean and standard error from an array (B, ...) of
    per-history batch means."""
    a = np.asarray(batch_doses, dtype=np.float64)
    return a.mean(0), a.std(0, ddof=1) / math.sqrt(len(a))


def _t_quantile(p, dof):
    from scipy import stats
    return stats.t.ppf(p, dof)


def compare(a, sa, ba, b, sb, bb, threshold=0.1):
    """Statistics of estimate a (mean, standard error, batch count) against b
    in the voxels whose dose exceeds `threshold` of the maximum dose.

    The voxels are chosen on the inverse-variance-weighted mean m of a and b,
    which (for normal noise) is independent of a - b: choosing them on b
    alone would keep the voxels where b's noise went up and bias a - b low by
    an amount that grows with b's noise. Relative differences are taken
    against m for the same reason.

    Returns a dict: voxels compared, the fraction within the t-corrected
    combined 2 sigma, the mean signed difference (dose-weighted: the summed
    difference over the summed dose; the plain mean of the per-voxel relative
    differences is given beside it), the mean |relative difference| and its
    excess over the statistical expectation (E|N(0,s)| = sqrt(2/pi) s per
    voxel), the largest |relative difference|, the ratio of the summed doses
    and its z-score."""
    a, sa, b, sb = (np.asarray(x, dtype=np.float64).reshape(-1) for x in (a, sa, b, sb))
    wa = 1.0 / np.maximum(sa * sa, 1e-300)
    wb = 1.0 / np.maximum(sb * sb, 1e-300)
    m = (wa * a + wb * b) / (wa + wb)
    mask = m > threshold * m.max()
    a, sa, b, sb, m = a[mask], sa[mask], b[mask], sb[mask], m[mask]
    s2 = sa * sa + sb * sb
    s = np.sqrt(s2)
    den = sa ** 4 / max(ba - 1, 1) + sb ** 4 / max(bb - 1, 1)
    dof = np.where(den > 0, s2 * s2 / np.maximum(den, 1e-300), 1e9)
    tq = _t_quantile(0.5 + 0.5 * P_2SIGMA, np.maximum(dof, 1.0))
    ok = np.abs(a - b) <= tq * s
    rel = (a - b) / m
    noise = math.sqrt(2.0 / math.pi) * s / m
    tot_a, tot_b = a.sum(), b.sum()
    tot_s = math.sqrt(float((sa ** 2).sum() + (sb ** 2).sum()))   # voxels treated as independent
    return {
        "voxels": int(mask.sum()),
        "within_2sigma": float(ok.mean()),
        "expected_within_2sigma": P_2SIGMA,
        "mean_signed_pct": 100.0 * float((tot_a - tot_b) / m.sum()),
        "mean_signed_voxel_pct": 100.0 * float(rel.mean()),
        "mean_abs_pct": 100.0 * float(np.abs(rel).mean()),
        "mean_abs_noise_pct": 100.0 * float(noise.mean()),
        "mean_abs_excess_pct": 100.0 * max(0.0, float(np.abs(rel).mean() - noise.mean())),
        "max_abs_pct": 100.0 * float(np.abs(rel).max()),
        "total_ratio": float(tot_a / tot_b),
        "total_z": float((tot_a - tot_b) / tot_s) if tot_s > 0 else 0.0,
        "mean_rel_sigma_pct": 100.0 * float((s / m).mean()),
    }
