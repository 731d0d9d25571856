"""The seeded generator behind every synthetic workload (CPU only)."""
import numpy as np
import pytest

from pascal_btdma_gb300 import synth


def test_philox4x32_10_known_answers():
    # Known-answer vectors published with Random123 (Salmon et al., SC'11), kat_vectors.
    assert synth.philox4x32_10((0, 0, 0, 0), (0, 0)) == (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)
    assert synth.philox4x32_10((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2) == (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)
    assert synth.philox4x32_10((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0)) == (
        0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)


def test_uniform_range_and_determinism():
    v = np.array([synth.uniform(42, 0, s, r, e) for s in range(8) for r in range(8) for e in range(9)])
    assert v.min() >= -1.0 and v.max() < 1.0
    assert abs(v.mean()) < 0.15 and 0.25 < v.var() < 0.42
    assert synth.uniform(42, 0, 3, 4, 5) == synth.uniform(42, 0, 3, 4, 5)
    assert synth.uniform(42, 0, 3, 4, 5) != synth.uniform(43, 0, 3, 4, 5)


def test_fill_independent_of_thread_count():
    a = synth.dominant(4, 37, 19, seed=5, delta=1.2, nthreads=1)
    b = synth.dominant(4, 37, 19, seed=5, delta=1.2, nthreads=7)
    for x, y in zip(a.arrays, b.arrays):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("delta", [1.05, 1.2, 2.0])
def test_dominant_structure(delta):
    m, nsys, N = 5, 16, 12
    w = synth.dominant(m, nsys, N, seed=1, delta=delta)
    A = w.A.reshape(m, m, N, nsys)  # [j, i, row, sys]
    B = w.B.reshape(m, m, N, nsys)
    Cm = w.C.reshape(m, m, N, nsys)
    assert np.all(A[:, :, 0, :] == 0) and np.all(Cm[:, :, N - 1, :] == 0)
    for i in range(m):
        off = np.abs(A[:, i]).sum(0) + np.abs(Cm[:, i]).sum(0) + np.abs(B[:, i]).sum(0) - np.abs(B[i, i])
        # B_ii = R_ii + delta*rowsum(|A|+|C|+|R|) dominates the rest of its row
        assert np.all(np.abs(B[i, i]) > off * (delta - 1.0) - 1e-12)


def test_row_scale_log_uniform():
    m, nsys, N = 3, 64, 32
    base = synth.dominant(m, nsys, N, seed=9, delta=1.5)
    sc = synth.dominant(m, nsys, N, seed=9, delta=1.5, row_scale=True)
    ratio = (sc.D / base.D).reshape(m, N, nsys)[0]
    assert ratio.min() >= 1e-3 * (1 - 1e-12) and ratio.max() <= 1e3 * (1 + 1e-12)
    l = np.log10(ratio).ravel()
    assert -0.3 < l.mean() < 0.3 and 1.6 < l.std() < 1.85  # uniform on [-3, 3]: mean 0, std sqrt(3)
    # the whole block row is scaled by the same factor
    assert np.allclose((sc.B / base.B).reshape(m, m, N, nsys)[1, 2], ratio, rtol=1e-14)


def test_exp2_deterministic_and_accurate():
    t = np.linspace(-20, 20, 1001)
    got = np.array([synth.N.synth_lib().pbt_synth_exp2(float(x)) for x in t])
    assert np.allclose(got, np.exp2(t), rtol=2e-15, atol=0)


def test_uneven_shapes():
    n, m = synth.uneven_shapes(11, 32768)
    assert n.min() >= 16 and n.max() <= 4096 and set(np.unique(m)) == {2, 3, 4, 5}
    l = np.log2(n)
    assert 6.5 < l.mean() < 8.5  # log-uniform on [4, 12]
    n2, m2 = synth.uneven_shapes(11, 32768)
    assert np.array_equal(n, n2) and np.array_equal(m, m2)


def test_fill_batch_matches_uniform_fill():
    """System s of a batch = system index s of a uniform batch with its shape."""
    m = np.array([3, 3, 5, 2], dtype=np.int32)
    n = np.array([7, 7, 4, 9], dtype=np.int32)
    A, B, Cc, D, mo, vo = synth.fill_batch(m, n, seed=21, delta=1.3, nthreads=3)
    for s in range(4):
        u = synth.dominant(int(m[s]), s + 1, int(n[s]), seed=21, delta=1.3)
        ms, ns = int(m[s]), int(n[s])
        ua = u.A.reshape(ms * ms * ns, s + 1)[:, s]
        ud = u.D.reshape(ms * ns, s + 1)[:, s]
        assert np.array_equal(A[mo[s]:mo[s] + ms * ms * ns], ua)
        assert np.array_equal(D[vo[s]:vo[s] + ms * ns], ud)
