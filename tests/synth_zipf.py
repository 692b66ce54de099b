"""Plain-Python restatement of the device generator of the load-imbalanced
synthetic workload (te_matrix_create_zipf in te_synth.cu), used by the tests
to check the GPU-built matrix entry by entry at small sizes.

Same counter-based hash, same draws, same merge order: the structure (row
pointers, columns) must agree exactly and the values up to the rounding of
the transcendental functions (Box-Muller) and of the power-iteration norms.
"""
import math

import numpy as np

MASK = (1 << 64) - 1


def mix64(z):
    z = (z + 0x9E3779B97F4A7C15) & MASK
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
    return z ^ (z >> 31)


def draw(seed, row, t, stream):
    return mix64(mix64(mix64(seed) ^ row) ^ (((t << 8) | stream) & MASK))


def unit_open_right(h):
    return (h >> 11) * 2.0 ** -53


def unit_open_left(h):
    return ((h >> 11) + 1) * 2.0 ** -53


def gaussian_pair(h1, h2):
    rad = math.sqrt(-2.0 * math.log(unit_open_left(h1)))
    u = unit_open_right(h2)
    return complex(rad * math.cos(2.0 * math.pi * u), rad * math.sin(2.0 * math.pi * u))


def zipf_cdf(exponent, min_len, max_len):
    z = 0.0
    cdf = []
    for k in range(min_len, max_len + 1):
        z += math.pow(k, -exponent)
        cdf.append(z)
    cdf = [c / z for c in cdf]
    cdf[-1] = 1.0
    return np.array(cdf)


def row_lengths(n, exponent, min_len, max_len, seed):
    cdf = zipf_cdf(exponent, min_len, max_len)
    u = np.array([unit_open_right(draw(seed, r, 0, 0)) for r in range(n)])
    return min_len + np.searchsorted(cdf, u, side="right")


def generate(n, exponent=1.5, min_len=2, max_len=256, seed=1, power_iters=30):
    """Returns (row_ptr, col, values, norm_estimate) of H = (A + A^H)/2 / estimate."""
    lens = row_lengths(n, exponent, min_len, max_len, seed)
    rows = []
    for r in range(n):
        cols = []
        for t in range(int(lens[r])):
            for a in range(64):
                c = draw(seed, r, a * 65536 + t, 1) % n
                if c not in cols:
                    break
            else:
                raise RuntimeError("no distinct column")
            cols.append(c)
        vals = [gaussian_pair(draw(seed, r, t, 2), draw(seed, r, t, 3)) for t in range(len(cols))]
        rows.append((cols, vals))
    own = [dict() for _ in range(n)]
    mirror = [dict() for _ in range(n)]
    for r, (cols, vals) in enumerate(rows):
        for c, v in zip(cols, vals):
            own[r][c] = v
            mirror[c][r] = v.conjugate()
    rp = [0]
    col, val = [], []
    for r in range(n):
        keys = sorted(set(own[r]) | set(mirror[r]))
        for c in keys:
            if c in own[r] and c in mirror[r]:
                s = own[r][c] + mirror[r][c]
            else:
                s = own[r].get(c, mirror[r].get(c))
            col.append(c)
            val.append(complex(0.5 * s.real, 0.5 * s.imag))
        rp.append(len(col))
    rp = np.array(rp, dtype=np.int64)
    col = np.array(col, dtype=np.int64)
    val = np.array(val, dtype=np.complex128)
    est = 1.0
    if power_iters > 0:
        import scipy.sparse as sp
        H = sp.csr_matrix((val, col, rp), shape=(n, n))
        x = np.array([gaussian_pair(draw(seed, r, 0, 4), draw(seed, r, 1, 4)) for r in range(n)])
        x /= np.linalg.norm(x)
        for _ in range(power_iters):
            y = H @ x
            est = np.linalg.norm(y)
            x = y / est
        val = val * (1.0 / est)
    return rp, col, val, est
