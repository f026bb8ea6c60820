"""Integrated autocorrelation time and effective sample counts.

The reference has no estimator of its own (its analysis lived in the external
origamipy package), so one is fixed here and applied identically to every
run: the normalised autocorrelation function of each series by FFT and
Sokal's automatic window (smallest M with M >= c * tau(M), c = 5)."""
import numpy as np


def tau_int(x, c=5.0):
    """Integrated autocorrelation time of a 1-D series, in samples, with the
    convention tau = 1/2 + sum_{k>=1} rho(k) (so iid data gives 1/2).
    Returns None for a constant series."""
    x = np.asarray(x, dtype=np.float64)
    n = len(x)
    if n < 4:
        return None
    x = x - x.mean()
    var = np.dot(x, x) / n
    if var <= 0:
        return None
    m = 1 << (2 * n - 1).bit_length()
    f = np.fft.rfft(x, m)
    acf = np.fft.irfft(f * np.conj(f), m)[:n] / (n * var)
    tau = 0.5
    for M in range(1, n):
        tau += acf[M]
        if M >= c * tau:
            return max(tau, 0.5)
    return max(tau, 0.5)


def effective_samples(series):
    """Sum over replicas of n / (2 tau).  A series that never changed carries
    one effective sample."""
    total = 0.0
    taus = []
    for s in series:
        t = tau_int(s)
        if t is None:
            total += 1.0
            continue
        taus.append(t)
        total += len(s) / (2.0 * t)
    return total, (float(np.median(taus)) if taus else None)


def replica_ess(series):
    """Effective samples of each replica's series, n / (2 tau) (one for a
    series that never changed)."""
    out = np.empty(len(series))
    for i, s in enumerate(series):
        t = tau_int(s)
        out[i] = 1.0 if t is None else len(s) / (2.0 * t)
    return out


def bootstrap_sum(per_replica, groups=None, n_boot=2000, seed=0, level=0.95):
    """Percentile bootstrap of a sum over independent replicas: replicas are
    resampled with replacement, within each group (e.g. scaffold size) if
    groups is given.  Returns (lo, hi) and the bootstrap sums."""
    x = np.asarray(per_replica, dtype=np.float64)
    rng = np.random.default_rng(seed)
    g = np.zeros(len(x), int) if groups is None else np.asarray(groups)
    sums = np.zeros(n_boot)
    for key in np.unique(g):
        idx = np.flatnonzero(g == key)
        pick = rng.integers(0, len(idx), size=(n_boot, len(idx)))
        sums += x[idx][pick].sum(axis=1)
    a = (1.0 - level) / 2.0
    return (float(np.quantile(sums, a)), float(np.quantile(sums, 1.0 - a))), sums


def tau_vs_length(series, lengths):
    """Median tau_int over replicas of the first L samples, for each L."""
    out = {}
    for L in lengths:
        ts = [tau_int(s[:L]) for s in series if len(s) >= L]
        ts = [t for t in ts if t is not None]
        out[int(L)] = float(np.median(ts)) if ts else None
    return out
