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
