"""Algorithmic operation counts of the GPU sieve, used for roofline figures.

Counts are multiply-adds (MACs) of the algorithm as the kernels run it, without the padding
and idle lanes of the warp mapping; one complex MAC is 8 real flops, one real MAC 2.

Per sieve term with an m x m term matrix (mb = m + border, rows = mb + odd-mode rows):
* Hessenberg reduction by Gaussian elimination, step j = 0..mb-2, L = mb-j-1:
    row scaling L, phase A (rows below the pivot) (L-1)*L, phase B (column update) rows*L
* La Budde's recurrence truncated to Kc = min(K, m) coefficients:
    sum_{i=1..m} sum_{j=1..min(i,Kc)} min(j, i)
* det^(-1/2) series to degree K: sum_{n=1..K} min(n, Kc)
* loop variants: the border series from La Budde's trailing determinants, per bordered row
  (1 + odd-mode rows) sum_{t=1..K} (min(t, Kc) + min(t-1, Kc)) (numerator, division by P), and
  the exp series K^2/2 (+ N^2/2 odd)

``reference_term_macs`` is the reference's own per-term work (charpoly.powertrace by repeated
matrix products, (K-1) * m^3 MACs), reported beside, never mixed into, the roofline.
"""
import numpy as np

__all__ = ["term_macs", "instance_flops", "plain_hafnian_flops", "reference_term_macs"]


def term_macs(m, K, border=0, extra_rows=0, loop=False, odd_N=0):
    mb = m + border
    rows = mb + extra_rows
    hess = 0
    for j in range(mb - 1):
        L = mb - j - 1
        hess += L + (L - 1) * L + rows * L
    Kc = min(K, m)
    lab = 0
    for i in range(1, m + 1):
        for j in range(1, min(i, Kc) + 1):
            lab += min(j, i)
    ser = sum(min(n, Kc) for n in range(1, K + 1))
    extra = 0
    if loop:
        extra += (1 + extra_rows) * sum(min(t, Kc) + min(t - 1, Kc) for t in range(1, K + 1)) + K * K // 2
        if odd_N:
            extra += odd_N * odd_N // 2
    return hess + lab + ser + extra


def _edge_m_distribution(edge_reps, glynn=True, half_first=True):
    """Histogram {number of nonzero-delta edges: term count} over the sieve's terms."""
    dist = {0: 1}
    for i, r in enumerate(edge_reps):
        r = int(r)
        digits = range((r + 2) // 2) if (i == 0 and half_first) else range(r + 1)
        nz = sum(1 for k in digits if ((2 * k - r) if glynn else k) != 0)
        z = len(digits) - nz
        new = {}
        for e, c in dist.items():
            if nz:
                new[e + 1] = new.get(e + 1, 0) + c * nz
            if z:
                new[e] = new.get(e, 0) + c * z
        dist = new
    return dist


def instance_flops(edge_reps, complex_input=True, kind="plain", glynn=True, odd=False):
    """Algorithmic flops of one sieve instance (sum over all terms)."""
    N = 2 * int(np.sum(edge_reps)) + (1 if odd else 0)
    K = N // 2
    half_first = glynn and not odd
    loop = kind != "plain"
    total = 0
    for e, cnt in _edge_m_distribution(edge_reps, glynn, half_first).items():
        total += cnt * term_macs(2 * e, K, border=1 if loop else 0, extra_rows=1 if odd else 0,
                                 loop=loop, odd_N=N if odd else 0)
    return total * (8 if complex_input else 2)


def plain_hafnian_flops(n, complex_input=True):
    """Flops of one plain Glynn hafnian of an n x n matrix (all repetitions 1)."""
    return instance_flops([1] * (n // 2), complex_input)


def reference_term_macs(m, K):
    """MACs of one term in the reference (powertrace by K-1 repeated m x m products)."""
    return max(K - 1, 0) * m**3
