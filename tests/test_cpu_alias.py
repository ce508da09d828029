"""Alias tables of the opt-in environment-light sampling mode (cpu).

rt_debug_alias returns the table the library builds for a Distribution1D CDF
(Distribution1D.cs:19-49).  The renderer's uniforms are u = k / 2^24 for
k in [0, 2^24) (NextFloat).  The alias pick (AliasPick in rt_shading.cuh:
bucket i = floor(k n / 2^24), kept when k n mod 2^24 is below the bucket's
threshold, else its alias) must select every entry for exactly as many k as
the reference's CDF search (FindInterval and SampleContinuous,
Distribution1D.cs:51-85) does: the same pmf, not an approximation of it.
Both pickers are enumerated over all 2^24 values of k with exact integer and
binary32-exact arithmetic.
"""
import numpy as np
import pytest

from radiantium_gb300 import native as N

K = 1 << 24


@pytest.fixture(scope="module")
def lib():
    return N.load_library()


def cdf_of(f):
    """Distribution1D's CDF in binary32, operation for operation (Distribution1D.cs:26-48)."""
    f = np.asarray(f, np.float32)
    n = f.size
    cdf = np.zeros(n + 1, np.float32)
    nn = np.float32(n)
    for i in range(1, n + 1):
        cdf[i] = np.float32(cdf[i - 1] + np.float32(f[i - 1] / nn))
    integ = cdf[n]
    if integ == 0:
        cdf[1:] = np.arange(1, n + 1, dtype=np.float32) / nn
    else:
        with np.errstate(invalid="ignore"):
            cdf[1:] = cdf[1:] / integ
    return cdf


def alias_table(lib, cdf):
    n = cdf.size - 1
    out = np.zeros((n, 2), np.int32)
    rc = lib.rt_debug_alias(np.ascontiguousarray(cdf).ctypes.data, n, out.ctypes.data)
    return rc, out


def counts_search(cdf):
    """How many k each entry gets from FindInterval: the last i with cdf[i] <= k / 2^24, clamped."""
    n = cdf.size - 1
    out = np.zeros(n, np.int64)
    c64 = cdf.astype(np.float64)
    for k0 in range(0, K, 1 << 22):
        u = np.arange(k0, k0 + (1 << 22), dtype=np.float64) / K
        i = np.clip(np.searchsorted(c64, u, side="right") - 1, 0, n - 1)
        out += np.bincount(i, minlength=n)
    return out


def counts_alias(tab):
    n = tab.shape[0]
    thr = tab[:, 0].astype(np.int64)
    ali = tab[:, 1].astype(np.int64)
    out = np.zeros(n, np.int64)
    for k0 in range(0, K, 1 << 22):
        s = np.arange(k0, k0 + (1 << 22), dtype=np.int64) * n
        i = s >> 24
        pick = np.where((s & (K - 1)) < thr[i], i, ali[i])
        out += np.bincount(pick, minlength=n)
    return out


def _env_row_weights(w, h, seed):
    """Luminance * sin(theta) of a lat-long map with a bright sun, dark bands and exact zeros."""
    rng = np.random.default_rng(seed)
    lum = rng.gamma(0.6, 1.0, (h, w)).astype(np.float32)
    lum[h // 3: h // 3 + 3, :] = 0
    lum[:, w // 5: w // 5 + 7] = 0
    lum[h // 4, w // 2] = 5e4
    s = np.sin((np.arange(h, dtype=np.float32) + np.float32(0.5)) / np.float32(h) * np.float32(3.14159265))
    return (lum * s[:, None].astype(np.float32)).astype(np.float32)


CASES = {
    "random_1024": lambda: np.random.default_rng(1).random(1024),
    "env_marginal_512": lambda: _env_row_weights(64, 512, 2).sum(1),
    "env_row_1000": lambda: _env_row_weights(1000, 8, 3)[1],
    "zeros_1000": lambda: np.zeros(1000),
    "one_spike_7": lambda: np.array([0, 0, 0, 3.5, 0, 0, 0]),
    "single_entry": lambda: np.array([2.0]),
    "heavy_tail_3001": lambda: np.random.default_rng(4).pareto(0.7, 3001),
    "tiny_values_333": lambda: np.random.default_rng(5).random(333) * 1e-30,
    "wide_row_8191": lambda: _env_row_weights(8191, 4, 6)[2],
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_alias_pick_draws_the_search_pmf_exactly(lib, name):
    f = np.asarray(CASES[name](), np.float32)
    cdf = cdf_of(f)
    rc, tab = alias_table(lib, cdf)
    assert rc == N.RT_OK
    n = f.size
    assert ((tab[:, 1] >= 0) & (tab[:, 1] < n)).all()
    assert ((tab[:, 0] >= 0) & (tab[:, 0].astype(np.int64) <= K + n)).all()
    want = counts_search(cdf)
    got = counts_alias(tab)
    assert want.sum() == K and got.sum() == K
    assert np.array_equal(got, want), (name, np.nonzero(got != want)[0][:10])


def test_alias_rejects_tables_the_search_cannot_treat_as_a_pmf(lib):
    for f in (np.array([1, -0.5, 2], np.float32), np.array([1, np.nan, 2], np.float32),
              np.array([1, np.inf, 2], np.float32)):
        rc, _ = alias_table(lib, cdf_of(f))
        assert rc == N.RT_ERR_UNSUPPORTED, f
    bad = np.array([0, 0.5, 0.4, 1], np.float32)
    assert alias_table(lib, bad)[0] == N.RT_ERR_UNSUPPORTED
    assert alias_table(lib, np.array([0, 0.5, 0.9], np.float32))[0] == N.RT_ERR_UNSUPPORTED
