"""The transport step that allocates nothing (psgb_transport_step_noalloc), against the
regular entry point (psgb_transport_step) on the same inputs.

It serves callers that may not call cudaMalloc while they run (a fixed memory budget,
code around stream capture or in a latency-critical loop): its workspace is the
library's static device scratch. This file is collected last on purpose, so a run that
stops at the first failure has already run every other test."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


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
        assert np.max(np.abs(tn - ref_t)) <= 2e-6
        assert np.max(np.abs(h - ref_h)) <= 2e-6 * inp.heat_capacity / inp.dt
        assert abs(rep.sum_W) <= 1e-13 * rep.absolute_sum_W


def test_no_alloc_step_rejects_planets_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    import planet_game_gb300 as pg

    m = pg.make_icosphere(6, 6.371e6)       # 40,962 cells > 10,242
    t = torch.zeros(m.cell_count, dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError, match="10242"):
        pg.api.transport_step_noalloc(m, t, t, 4e7, 2.6e6, 4e13)
