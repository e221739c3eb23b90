"""The L8 multi-right-hand-side case: one 655,362-cell planet, 32 sub-steps with sources
S_j = S + N(0, 5^2) W/m^2, solved as one block (psgb_transport_step_multi: the matrix
read once per sweep for all 32), in plain FP64 (variant A) and with the FP32 inner solve
inside FP64 refinement (variant B).

Bars: every sub-step meets ||b - A x|| <= 1e-10 ||b|| and closure <= 1e-12; every
sub-step's new temperature and transport are bit-identical to the same sub-step solved
alone (psgb_transport_step); the two variants agree to 1e-6 K; all 32 agree with the FP64
CPU oracle (PCG + SGS V-cycle to 1e-13) to 2e-6 K, the transport step's bar."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

RHS = 32


@pytest.fixture(scope="module")
def l8():
    import planet_game_gb300 as pg
    from planet_game_gb300 import workloads as W

    m = pg.make_icosphere(8, 6.371e6)
    inp = W.step_inputs(m, seed=8)
    sources = W.perturbed_sources(inp.source, RHS, seed=9)
    return m, inp, sources


@pytest.fixture(scope="module")
def blocks(l8):
    torch = pytest.importorskip("torch")
    import planet_game_gb300 as pg

    m, inp, sources = l8
    t0 = torch.from_numpy(inp.t0).cuda()
    src = [torch.from_numpy(np.ascontiguousarray(s)).cuda() for s in sources]
    out = {}
    for precision in ("fp64", "mixed"):
        t, h, reps = pg.transport_step_multi(m, t0, src, inp.heat_capacity, inp.dt, inp.conductance,
                                             transport=True, precision=precision)
        torch.cuda.synchronize()
        out[precision] = ([x.cpu().numpy() for x in t], [x.cpu().numpy() for x in h], reps)
    return t0, src, out


def test_block_meets_the_gates_and_the_variants_agree(blocks):
    _, _, out = blocks
    for precision, (t, h, reps) in out.items():
        for r in reps:
            assert r.status == 0 and r.relative_residual <= 1e-10 and r.closure <= 1e-12, (precision, r)
            assert abs(r.sum_W) <= 1e-13 * r.absolute_sum_W
    ta, tb = np.array(out["fp64"][0]), np.array(out["mixed"][0])
    assert np.max(np.abs(ta - tb)) <= 1e-6
    assert all(r.refinements >= 2 for r in out["mixed"][2])        # FP32 inner: refinement at work


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_every_block_sub_step_equals_the_sub_step_alone(l8, blocks, precision):
    import planet_game_gb300 as pg

    m, inp, _ = l8
    t0, src, out = blocks
    t, h, reps = out[precision]
    for j in range(RHS):
        t1, h1, r1 = pg.transport_step(m, t0, src[j], inp.heat_capacity, inp.dt, inp.conductance,
                                       precision=precision)
        assert np.array_equal(t[j], t1.cpu().numpy()), j
        assert np.array_equal(h[j], h1.cpu().numpy()), j
        assert (reps[j].iterations, reps[j].refinements) == (r1.iterations, r1.refinements)
        assert reps[j].relative_residual == r1.relative_residual


def test_all_32_sub_steps_against_the_oracle(l8, blocks):
    m, inp, sources = l8
    _, _, out = blocks
    refs = O.transport_steps(m.arrays(), inp.conductance, inp.heat_capacity, inp.dt, [inp.t0] * RHS,
                             [np.ascontiguousarray(s) for s in sources], tol=1e-13)
    for j, (t_new, _, _) in enumerate(refs):
        assert np.max(np.abs(out["fp64"][0][j] - t_new)) <= 2e-6, j
        assert np.max(np.abs(out["mixed"][0][j] - t_new)) <= 2e-6, j


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_tuned_block_with_block_sweeps_equals_the_tuned_sub_steps_alone(l8, precision):
    """With per-level settings on the planet (block-local sweeps on the coarse levels, the
    coarse-grid correction scaled, ω = 1), the block step's sub-steps still equal the same
    sub-steps solved alone with those settings, bit for bit."""
    torch = pytest.importorskip("torch")
    import planet_game_gb300 as pg

    m, inp, sources = l8
    t = m.tuning
    depth = t["levels"]
    t.update(pre_sweeps=[1] + [2] * (depth - 1), post_sweeps=[2] + [2] * (depth - 1),
             block_sweeps=[1] + [6] * (depth - 1), jacobi_omega=1.0, coarse_correction=1.5)
    m.set_tuning(t)
    try:
        assert m.tuning["block_sweeps"][1] == 6 and m.tuning["coarse_correction"] == 1.5
        t0 = torch.from_numpy(inp.t0).cuda()
        src = [torch.from_numpy(np.ascontiguousarray(s)).cuda() for s in sources[:8]]
        tb, hb, rb = pg.transport_step_multi(m, t0, src, inp.heat_capacity, inp.dt, inp.conductance,
                                             transport=True, precision=precision)
        torch.cuda.synchronize()
        for j in range(len(src)):
            assert rb[j].status == 0 and rb[j].relative_residual <= 1e-10
            t1, h1, r1 = pg.transport_step(m, t0, src[j], inp.heat_capacity, inp.dt, inp.conductance,
                                           precision=precision)
            assert np.array_equal(tb[j].cpu().numpy(), t1.cpu().numpy()), j
            assert np.array_equal(hb[j].cpu().numpy(), h1.cpu().numpy()), j
            assert (rb[j].iterations, rb[j].refinements) == (r1.iterations, r1.refinements)
    finally:
        m.set_tuning(None)
    assert m.tuning["coarse_correction"] == 1.0
