"""Per-problem constant tables, built on the host exactly as the reference
builds them (``SingleScatterSimulationTOF.py:99-150``) and handed to the GPU.

* detector energy efficiency (SciPy ``erf``, the reference's own call) and
  the water attenuation ratio per 0.5 keV energy row;
* the TOF weight table, reduced to what the kernel evaluates: for each of
  the 8001 integer offsets the bin with the largest normalised weight and
  the base-2 log of that weight.  The kernel rebuilds every bin's weight
  from it with the Gaussian's closed-form ratio between bins.
"""

from __future__ import annotations

import numpy as np

ENERGY_REFERENCE = 511
TOF_TIME_RANGE = 4000


def energy_reference_row(att_table: np.ndarray) -> int:
    rows = np.where(att_table[:, 0] == ENERGY_REFERENCE)[0]
    if len(rows) != 1:
        raise ValueError("attenuation table has no unique 511 keV row")
    return int(rows[0])


def efficiency(energies: np.ndarray, threshold: float, resolution: float) -> np.ndarray:
    """0.5*(1 - erf((Eth - E) / (511*ER/2/sqrt(ln 2)))) (:139-140)."""
    from scipy.special import erf

    return 0.5 * (1 - erf((threshold - energies) /
                          (ENERGY_REFERENCE * resolution / 2 / np.sqrt(np.log(2)))))


def attenuation_ratio(att_table: np.ndarray) -> np.ndarray:
    """Water mu(E) / mu(511 keV) (:117-120)."""
    ei = energy_reference_row(att_table)
    return att_table[:, 1] / att_table[ei, 1]


def pair_efficiency_f32(att_table: np.ndarray, threshold: float, resolution: float) -> np.ndarray:
    """eff(E) * eff(511 keV) per energy row as float32, with exact zeros where
    the FP64 product is zero (the reference skips those pairs, :505-509) and
    tiny non-zero products kept non-zero."""
    eff = efficiency(att_table[:, 0], threshold, resolution)
    prod = eff * eff[ENERGY_REFERENCE * 2 - 1]
    out = prod.astype(np.float32)
    tiny = (prod != 0) & (out == 0)
    out[tiny] = np.float32(np.finfo(np.float32).tiny)
    return out


def tof_table(nbins: int, tof_range: float, resolution: float) -> np.ndarray:
    """The reference's TOF efficiency table [nbins, 8001] (:142-150, :261-295)."""
    offset = np.arange(-TOF_TIME_RANGE, TOF_TIME_RANGE + 1)
    bw = 2 * tof_range / nbins
    shifts = ((np.arange(1, nbins + 1) - (nbins + 1) / 2) * bw).reshape(-1, 1)
    prob = offset.reshape(1, -1) - shifts
    prob = np.exp(-(prob ** 2) / (resolution ** 2 / 4 / np.log(2)))
    total = np.sum(prob, axis=0)
    zero = total == 0
    with np.errstate(invalid="ignore", divide="ignore"):
        prob = prob / total
    prob[:, zero] = 0
    return prob


def tof_log2_table(nbins: int, tof_range: float, resolution: float) -> np.ndarray:
    """float32 [8001, 2]: (log2 of the largest weight, its bin); -inf, 0 where
    the reference's column is all zero."""
    T = tof_table(nbins, tof_range, resolution)
    n = np.argmax(T, axis=0)
    top = T[n, np.arange(T.shape[1])]
    out = np.zeros((T.shape[1], 2), dtype=np.float32)
    with np.errstate(divide="ignore"):
        out[:, 0] = np.where(top > 0, np.log2(np.where(top > 0, top, 1.0)), -np.inf)
    out[:, 1] = n.astype(np.float32)
    return out


def tof_weights_from_log2(log2w: np.ndarray, nbins: int, tof_range: float,
                          resolution: float) -> np.ndarray:
    """The weights the kernel evaluates, in FP64 (used by the tests)."""
    bw = 2 * tof_range / nbins
    s0 = (1 - (nbins + 1) / 2) * bw
    kappa = 4.0 / resolution ** 2
    t = np.arange(-TOF_TIME_RANGE, TOF_TIME_RANGE + 1, dtype=np.float64)
    Y = log2w[:, 0].astype(np.float64)
    n = log2w[:, 1].astype(np.float64)
    delta = t - (s0 + n * bw)
    beta = 2 * kappa * bw * delta
    gamma = kappa * bw * bw
    b = np.arange(nbins, dtype=np.float64)[:, None]
    d = n[None, :] - b
    with np.errstate(invalid="ignore"):
        e = Y[None, :] - d * (beta[None, :] + gamma * d)
    return np.exp2(e)
