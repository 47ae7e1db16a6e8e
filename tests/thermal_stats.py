"""Equilibrium statistics of a sampled time series with batch-means standard errors (used by the
thermal-statistics fixtures and their GPU test)."""
import numpy as np


def batch_stats(x, n_batches=20):
    """Mean of x and its standard error from n_batches contiguous batch means (correlated samples)."""
    x = np.asarray(x, dtype=np.float64)
    n = len(x) // n_batches * n_batches
    b = x[:n].reshape(n_batches, -1).mean(axis=1)
    return float(x.mean()), float(b.std(ddof=1) / np.sqrt(n_batches))


def series_stats(E, mz, nos):
    """<m_z>, <E>/N and var(E)/N (each with its standard error) of a series of samples."""
    mz_m, mz_e = batch_stats(mz)
    e_m, e_e = batch_stats(np.asarray(E) / nos)
    d2 = (np.asarray(E) - np.mean(E)) ** 2 / nos
    v_m, v_e = batch_stats(d2)
    return {"mz": (mz_m, mz_e), "e": (e_m, e_e), "var_e": (v_m, v_e)}


def langevin(x):
    return 1.0 / np.tanh(x) - 1.0 / x
