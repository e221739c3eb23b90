"""The oracle's restatement of the GB300 V-cycle (damped Jacobi, aggregation, dense
coarsest solve) with a scaled coarse-grid correction, against the same V-cycle written
here with numpy/scipy on the oracle's own hierarchy (CPU)."""
import numpy as np
import pytest

scipy_sparse = pytest.importorskip("scipy.sparse")


def _numpy_vcycle(h, rhs, pre, post, omega, correction):
    levels = []
    for l in range(h.levels()):
        lv = h.level(l)
        d, o = h.values(l)
        n = lv["rows"]
        rows = np.repeat(np.arange(n), np.diff(lv["offset"].astype(np.int64)))
        off = scipy_sparse.csr_matrix((o, (rows, lv["column"].astype(np.int64))), shape=(n, n))
        levels.append((off, d, lv["aggregate"].astype(np.int64), n))

    def cycle(l, b):
        off, d, agg, n = levels[l]
        if l == len(levels) - 1:
            return np.linalg.solve((off + scipy_sparse.diags(d)).toarray(), b)
        x = omega * b / d
        for _ in range(pre - 1):
            x = x + omega * ((b - off @ x) / d - x)
        r = b - d * x - off @ x
        xc = cycle(l + 1, np.bincount(agg, weights=r, minlength=levels[l + 1][3]))
        x = x + correction * xc[agg]
        for _ in range(post):
            x = x + omega * ((b - off @ x) / d - x)
        return x

    return cycle(0, rhs)


@pytest.mark.parametrize("correction", [1.0, 1.5, 2.0])
def test_scaled_coarse_correction_vcycle(meshes, correction):
    from oracle import oracle as O

    m = meshes(4)
    a = m.arrays()
    s, K = 2.6e6 / 4e7, 4e13
    h = O.OracleHierarchy(O.OracleMesh(a))
    h.set_matrix(a["area_m2"] / s + K * a["graph_weight_sum"], -K * a["graph_weight"])
    rhs = np.random.default_rng(5).standard_normal(m.cell_count) * 1e12
    got = h.vcycle_jacobi(rhs, 2, 2, 0.8, correction)
    want = _numpy_vcycle(h, rhs, 2, 2, 0.8, correction)
    assert np.max(np.abs(got - want)) <= 1e-11 * np.max(np.abs(want))
    if correction == 1.0:
        assert np.array_equal(got, h.vcycle_jacobi(rhs, 2, 2, 0.8))
    else:
        assert not np.allclose(got, h.vcycle_jacobi(rhs, 2, 2, 0.8), rtol=1e-6)
