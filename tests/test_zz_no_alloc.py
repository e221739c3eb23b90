"""The transport step that allocates nothing (psgb_transport_step_noalloc), against the
regular entry point (psgb_transport_step) on the same inputs.

It serves callers that may not call cudaMalloc while they run: a loop that reserved a
fixed memory budget up front, a host that lends the library a GPU under a hard memory
cap, a plugin host whose own allocator owns the device memory. Its workspace is the
library's static device scratch; the arithmetic is the regular step's (same kernels, same
layout, same reduction order), so the results are compared bit for bit. This file is
collected last on purpose, so a run that stops at the first failure has already run every
other test."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _same(a, b):
    return np.array_equal(np.asarray(a), np.asarray(b))


def test_no_alloc_step_matches_the_regular_step_on_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    import planet_game_gb300 as pg
    from planet_game_gb300 import workloads as W

    m = pg.make_icosphere(5, 5.2e6)        # a fresh planet: nothing on the device yet
    assert m.device_bytes() == 0
    runs = []
    for seed in (1, 2):                      # two calls in a row, different inputs
        inp = W.step_inputs(m, seed=seed)
        t0 = torch.from_numpy(inp.t0).cuda()
        src = torch.from_numpy(inp.source).cuda()
        for precision in ("mixed", "fp64"):
            tn, h, rep = pg.api.transport_step_noalloc(m, t0, src, inp.heat_capacity, inp.dt, inp.conductance,
                                                       precision=precision)
            torch.cuda.synchronize()
            assert rep.status == 0 and rep.relative_residual <= 1e-10 and rep.closure <= 1e-12
            runs.append((inp, precision, tn.cpu().numpy(), h.cpu().numpy(), rep))
    # the no-allocation calls left the planet's own device footprint untouched
    assert m.device_bytes() == 0
    for inp, precision, tn, h, rep in runs:
        ref_t, ref_h, ref_rep = pg.transport_step(m, inp.t0, inp.source, inp.heat_capacity, inp.dt, inp.conductance,
                                                  precision=precision)
        assert ref_rep.status == 0
        assert _same(tn, ref_t) and _same(h, ref_h)
        assert (rep.iterations, rep.refinements) == (ref_rep.iterations, ref_rep.refinements)
        assert rep.relative_residual == ref_rep.relative_residual and rep.closure == ref_rep.closure
        assert abs(rep.sum_W) <= 1e-13 * rep.absolute_sum_W


def test_no_alloc_step_with_per_edge_conductance_at_its_largest_level():
    torch = pytest.importorskip("torch")
    import planet_game_gb300 as pg
    from planet_game_gb300 import workloads as W

    m = pg.make_icosphere(5, 7.1e6)        # 10,242 cells: the largest planet the scratch holds
    kappa = W.lognormal_edge_diffusivity(m.edge_count, seed=11)
    inp = W.step_inputs(m, seed=12, edge_diffusivity=kappa)
    t0 = torch.from_numpy(inp.t0).cuda()
    src = torch.from_numpy(inp.source).cuda()
    for _ in range(2):
        tn, h, rep = pg.api.transport_step_noalloc(m, t0, src, inp.heat_capacity, inp.dt, inp.conductance,
                                                   edge_conductance=inp.edge_conductance, precision="mixed")
        torch.cuda.synchronize()
        assert rep.status == 0 and rep.relative_residual <= 1e-10 and rep.closure <= 1e-12
        ref_t, ref_h, ref_rep = pg.transport_step(m, inp.t0, inp.source, inp.heat_capacity, inp.dt,
                                                  inp.conductance, edge_conductance=inp.edge_conductance,
                                                  precision="mixed")
        assert _same(tn.cpu().numpy(), ref_t) and _same(h.cpu().numpy(), ref_h)
        assert rep.iterations == ref_rep.iterations


def test_no_alloc_step_rejects_planets_beyond_its_scratch_and_bad_arrays():
    torch = pytest.importorskip("torch")
    import planet_game_gb300 as pg

    m = pg.make_icosphere(6, 6.371e6)       # 40,962 cells > 10,242
    t = torch.zeros(m.cell_count, dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError, match="10242"):
        pg.api.transport_step_noalloc(m, t, t, 4e7, 2.6e6, 4e13)
    m5 = pg.make_icosphere(5, 6.371e6)
    good = torch.full((m5.cell_count,), 280.0, dtype=torch.float64, device="cuda")
    for bad in (good.float(), good[:-1].clone(), good.cpu()):
        with pytest.raises(ValueError):
            pg.api.transport_step_noalloc(m5, bad, good, 4e7, 2.6e6, 4e13)
        with pytest.raises(ValueError):
            pg.api.transport_step_noalloc(m5, good, bad, 4e7, 2.6e6, 4e13)
    with pytest.raises(ValueError, match="stored"):
        pg.api.transport_step_noalloc(m5, good, good, 4e7, 2.6e6, edge_conductance="stored")
    # the C entry point itself refuses the stored conductance (it has none)
    import ctypes as C

    from planet_game_gb300 import capi

    params = capi.StepParams(4e7, 2.6e6, 0.0, None, 1)
    out = torch.empty_like(good)
    code = capi.load().psgb_transport_step_noalloc(
        m5.handle, C.byref(params), C.byref(pg.api.solve_options()), C.c_void_p(good.data_ptr()),
        C.c_void_p(good.data_ptr()), C.c_void_p(out.data_ptr()), None, C.byref(capi.StepReport()),
        C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert code == capi.ERR_INVALID_ARGUMENT
    assert "noalloc" in capi.load().psgb_last_error().decode()
