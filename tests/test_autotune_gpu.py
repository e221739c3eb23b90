"""The per-level autotuner: launch shapes never change a result, tuned sweeps still meet
the 1e-10 residual and 1e-12 closure gates, and a tuning carries over between batches of
the same planets bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def planets(meshes):
    from planet_game_gb300 import workloads as W

    specs = [(6, 8.1e6), (4, 3.3e6), (5, 6.0e6), (7, 5.0e6), (5, 4.1e6)]
    ms = [meshes(l, r) for l, r in specs]
    inputs = [W.step_inputs(m, seed=40 + i, edge_diffusivity=W.lognormal_edge_diffusivity(m.edge_count, 400 + i))
              for i, m in enumerate(ms)]
    return ms, inputs


def step(batch, inputs, **options):
    return batch.transport_step([i.t0 for i in inputs], [i.source for i in inputs], 4e7, inputs[0].dt,
                                edge_conductance=[i.edge_conductance for i in inputs], **options)


def test_autotune_meets_the_gates_and_carries_over(planets):
    import planet_game_gb300 as pg

    ms, inputs = planets
    batch = pg.Batch(ms)
    tuning = batch.autotune([i.t0 for i in inputs], [i.source for i in inputs], 4e7, inputs[0].dt,
                            edge_conductance=[i.edge_conductance for i in inputs], precision="mixed")
    depth = tuning["levels"]
    assert depth == len(ms[3].level_rows)
    assert all(1 <= p <= 8 for p in tuning["pre_sweeps"]) and all(0 <= p <= 8 for p in tuning["post_sweeps"])
    assert set(tuning["stencil_tiles"]) <= {1, 2} and set(tuning["vector_tiles"]) <= {1, 4}
    assert tuning["trial_solves"] >= 4 and tuning["tuned_solve_ms"] > 0
    assert tuning["tuned_solve_ms"] <= 1.25 * tuning["default_solve_ms"]
    assert batch.tuning["pre_sweeps"] == tuning["pre_sweeps"]
    out, reps = step(batch, inputs, precision="mixed")
    for r in reps:
        assert r.status == 0 and r.relative_residual <= 1e-10 and r.closure <= 1e-12
    # the same settings on a fresh batch of the same planets: identical results
    other = pg.Batch(ms)
    other.set_tuning(tuning)
    out2, reps2 = step(other, inputs, precision="mixed")
    for a, b, ra, rb in zip(out, out2, reps, reps2):
        assert np.array_equal(a, b) and ra.iterations == rb.iterations


def test_launch_shapes_never_change_results(planets):
    import planet_game_gb300 as pg

    ms, inputs = planets
    batch = pg.Batch(ms)
    base = batch.tuning
    outs = []
    for stencil, vector in ((1, 1), (2, 4), (2, 1), (1, 4)):
        t = dict(base)
        t["stencil_tiles"] = [stencil] * base["levels"]
        t["vector_tiles"] = [vector] * base["levels"]
        batch.set_tuning(t)
        for precision in ("mixed", "fp64"):
            out, reps = step(batch, inputs, precision=precision)
            assert all(r.status == 0 for r in reps)
            outs.append((precision, out))
    for precision in ("mixed", "fp64"):
        ref = [o for p, o in outs if p == precision]
        for other in ref[1:]:
            assert all(np.array_equal(a, b) for a, b in zip(ref[0], other))


def test_clearing_a_tuning_restores_the_option_sweeps(planets):
    import planet_game_gb300 as pg

    ms, inputs = planets
    plain = pg.Batch(ms)
    ref, _ = step(plain, inputs, precision="mixed", pre_sweeps=1, post_sweeps=1, jacobi_omega=1.0)
    batch = pg.Batch(ms)
    t = batch.tuning
    t["pre_sweeps"] = [3] * t["levels"]
    t["post_sweeps"] = [3] * t["levels"]
    batch.set_tuning(t)
    tuned, reps = step(batch, inputs, precision="mixed", pre_sweeps=1, post_sweeps=1, jacobi_omega=1.0)
    assert all(r.status == 0 for r in reps)
    assert not all(np.array_equal(a, b) for a, b in zip(ref, tuned))     # the tuning took precedence
    batch.set_tuning(None)
    back, _ = step(batch, inputs, precision="mixed", pre_sweeps=1, post_sweeps=1, jacobi_omega=1.0)
    assert all(np.array_equal(a, b) for a, b in zip(ref, back))
    bad = dict(t)
    bad["stencil_tiles"] = [3] * t["levels"]
    with pytest.raises(ValueError, match="tile sets"):
        batch.set_tuning(bad)


def test_coarse_tail_never_changes_results(planets):
    """The coarse levels run as one block per planet from any tail level, or grid-wide:
    the same phases in the same order per planet, so every result is bit-identical."""
    import planet_game_gb300 as pg

    ms, inputs = planets
    batch = pg.Batch(ms)
    base = batch.tuning
    assert base["coarse_tail_level"] >= 1              # chosen by the planets' level sizes
    for precision, method in (("mixed", "bicgstab"), ("fp64", "pcg")):
        outs = []
        for tail in range(base["levels"]):
            t = dict(base)
            t["coarse_tail_level"] = tail
            batch.set_tuning(t)
            out, reps = step(batch, inputs, precision=precision, method=method)
            assert all(r.status == 0 for r in reps)
            outs.append((out, [r.iterations for r in reps]))
        for out, its in outs[1:]:
            assert its == outs[0][1]
            assert all(np.array_equal(a, b) for a, b in zip(outs[0][0], out))


def test_block_sweeps_are_schedule_independent(planets):
    """Block-local sweeps (several Jacobi sweeps of a tile per launch, the tile's neighbours
    in other tiles held) give the same bits grid-wide, in the coarse tail at any level and
    in the persistent kernel, and the solves meet the gates."""
    import planet_game_gb300 as pg

    ms, inputs = planets
    batch = pg.Batch(ms)
    t = batch.tuning
    depth = t["levels"]
    t["pre_sweeps"] = [2] + [3] * (depth - 1)
    t["post_sweeps"] = [2] + [3] * (depth - 1)
    t["block_sweeps"] = [2] + [3] * (depth - 1)
    runs = []
    for tail in range(depth):
        t["coarse_tail_level"] = tail
        batch.set_tuning(t)
        for schedule in ("kernels", "persistent"):
            out, reps = step(batch, inputs, precision="mixed", schedule=schedule)
            for r in reps:
                assert r.status == 0 and r.relative_residual <= 1e-10 and r.closure <= 1e-12
            runs.append((out, [r.iterations for r in reps]))
    for out, its in runs[1:]:
        assert its == runs[0][1]
        assert all(np.array_equal(a, b) for a, b in zip(runs[0][0], out))


def test_spread_coarse_tail_equals_single_block_tail(planets):
    """Large planets' tails on several co-resident blocks (per-planet barriers) give the
    same bits as one block per planet and as no tail, in both precisions."""
    import planet_game_gb300 as pg

    ms, inputs = planets
    batch = pg.Batch(ms)
    t = batch.tuning
    for precision, method in (("mixed", "bicgstab"), ("fp64", "pcg")):
        runs = []
        for tail, single in ((0, 0), (1, 1), (1, 0), (2, 0)):
            t["coarse_tail_level"], t["coarse_tail_single"] = tail, single
            batch.set_tuning(t)
            out, reps = step(batch, inputs, precision=precision, method=method)
            assert all(r.status == 0 for r in reps)
            runs.append((out, [r.iterations for r in reps], batch.tuning["coarse_tail_blocks"]))
        assert runs[2][2] > len(ms)            # the L7 and L6 planets took several blocks
        for out, its, _ in runs[1:]:
            assert its == runs[0][1]
            assert all(np.array_equal(a, b) for a, b in zip(runs[0][0], out))


def test_shared_memory_coarse_tail_equals_no_tail(planets):
    """The tail with its levels' vectors in shared memory (one block per planet) gives the
    same bits as no tail at every tail level that fits, with plain and block-local sweeps,
    in both precisions."""
    import planet_game_gb300 as pg

    ms, inputs = planets
    batch = pg.Batch(ms)
    t = batch.tuning
    depth = t["levels"]
    for block in (1, 4):
        t["block_sweeps"] = [1] + [block] * (depth - 1)
        for precision, method in (("mixed", "bicgstab"), ("fp64", "pcg")):
            runs = []
            for tail, mode in [(0, 0)] + [(l, 2) for l in range(1, depth)]:
                t["coarse_tail_level"], t["coarse_tail_single"] = tail, mode
                batch.set_tuning(t)
                out, reps = step(batch, inputs, precision=precision, method=method)
                for r in reps:
                    assert r.status == 0 and r.relative_residual <= 1e-10
                runs.append((out, [r.iterations for r in reps]))
            for out, its in runs[1:]:
                assert its == runs[0][1]
                assert all(np.array_equal(a, b) for a, b in zip(runs[0][0], out))


def test_cluster_coarse_tail_equals_no_tail(planets):
    """The tail on a thread-block cluster of 2, 4 or 8 blocks per planet, the levels'
    vectors spread over the cluster's distributed shared memory, gives the same bits as no
    tail at every tail level and cluster size that fit, with plain and block-local sweeps,
    in both precisions; tails that do not fit fall back to another form, same bits."""
    import planet_game_gb300 as pg

    ms, inputs = planets
    batch = pg.Batch(ms)
    t = batch.tuning
    depth = t["levels"]
    for block in (1, 4):
        t["block_sweeps"] = [1] + [block] * (depth - 1)
        for precision, method in (("mixed", "bicgstab"), ("fp64", "pcg")):
            runs, clustered = [], set()
            for tail, mode, cluster in [(0, 0, 0)] + [(l, 3, c) for l in range(1, depth) for c in (2, 4, 8)]:
                t["coarse_tail_level"], t["coarse_tail_single"], t["coarse_tail_cluster"] = tail, mode, cluster
                batch.set_tuning(t)
                out, reps = step(batch, inputs, precision=precision, method=method)
                for r in reps:
                    assert r.status == 0 and r.relative_residual <= 1e-10
                got = batch.tuning
                assert got["coarse_tail_single"] == mode and got["coarse_tail_cluster"] == cluster
                if cluster and got["coarse_tail_blocks"] == len(ms) * cluster:
                    clustered.add((tail, cluster))
                runs.append((out, [r.iterations for r in reps]))
            # every cluster size ran from the coarsest tail levels at least
            assert {c for _, c in clustered} == {2, 4, 8}
            for out, its in runs[1:]:
                assert its == runs[0][1]
                assert all(np.array_equal(a, b) for a, b in zip(runs[0][0], out))


def test_cluster_tail_settings_are_checked(planets):
    import planet_game_gb300 as pg

    ms, _ = planets
    batch = pg.Batch(ms)
    t = batch.tuning
    t["coarse_tail_level"], t["coarse_tail_single"] = 1, 3
    for bad in (0, 1, 3, 16):
        t["coarse_tail_cluster"] = bad
        with pytest.raises(Exception, match="coarse_tail_cluster"):
            batch.set_tuning(t)


def test_shared_memory_tails_on_many_planets_stay_within_each_planet(meshes):
    """Twelve L5 planets: the later planets' coarse rows start far past their own slices
    of the shared-memory tails, so a load through a padding row's aggregate index that
    left the planet would fall outside the block's shared memory. Padding rows point at
    their own planet's first coarse row; the shared-memory and cluster tails give the
    same bits as no tail at every tail level, in both precisions."""
    import planet_game_gb300 as pg
    from planet_game_gb300 import workloads as W

    ms = [meshes(5, 4.0e6 + 2.5e5 * i) for i in range(12)]
    inputs = [W.step_inputs(m, seed=70 + i, edge_diffusivity=W.lognormal_edge_diffusivity(m.edge_count, 700 + i))
              for i, m in enumerate(ms)]
    batch = pg.Batch(ms)
    t = batch.tuning
    depth = t["levels"]
    for precision, method in (("mixed", "bicgstab"), ("fp64", "pcg")):
        runs = []
        forms = [(0, 0, 0)] + [(l, 2, 0) for l in range(1, depth)] + [(l, 3, c) for l in range(1, depth) for c in (2, 8)]
        for tail, mode, cluster in forms:
            t["coarse_tail_level"], t["coarse_tail_single"], t["coarse_tail_cluster"] = tail, mode, cluster
            batch.set_tuning(t)
            out, reps = step(batch, inputs, precision=precision, method=method)
            assert all(r.status == 0 and r.relative_residual <= 1e-10 for r in reps)
            if cluster:
                assert batch.tuning["coarse_tail_blocks"] == len(ms) * cluster
            runs.append((out, [r.iterations for r in reps]))
        for out, its in runs[1:]:
            assert its == runs[0][1]
            assert all(np.array_equal(a, b) for a, b in zip(runs[0][0], out))


def test_scaled_coarse_correction_same_bits_on_every_schedule_and_meets_the_oracle(planets):
    """With the V-cycle's coarse-grid correction scaled (over-correction, 1.5 and 2), every
    tail form and the persistent schedule give the kernel schedule's bits, in both
    precisions, and every planet's step meets the oracle's FP64 solve within 2e-6 K."""
    import planet_game_gb300 as pg
    from oracle import oracle as O

    ms, inputs = planets
    batch = pg.Batch(ms)
    t = batch.tuning
    for correction in (1.5, 2.0):
        t["coarse_correction"] = correction
        for precision, method in (("mixed", "bicgstab"), ("fp64", "pcg")):
            runs = []
            for tail, mode, cluster in ((0, 0, 0), (1, 1, 0), (1, 0, 0), (1, 2, 0), (1, 3, 4), (2, 2, 0)):
                t["coarse_tail_level"], t["coarse_tail_single"], t["coarse_tail_cluster"] = tail, mode, cluster
                batch.set_tuning(t)
                assert batch.tuning["coarse_correction"] == correction
                out, reps = step(batch, inputs, precision=precision, method=method)
                assert all(r.status == 0 and r.relative_residual <= 1e-10 and r.closure <= 1e-12 for r in reps)
                runs.append((out, [r.iterations for r in reps]))
            t["coarse_tail_level"], t["coarse_tail_single"], t["coarse_tail_cluster"] = 0, 0, 0
            batch.set_tuning(t)
            out, reps = step(batch, inputs, precision=precision, method=method, schedule="persistent")
            runs.append((out, [r.iterations for r in reps]))
            for out, its in runs[1:]:
                assert its == runs[0][1]
                assert all(np.array_equal(a, b) for a, b in zip(runs[0][0], out))
            if correction == 2.0 and precision == "mixed":
                for m, inp, got in zip(ms, inputs, runs[0][0]):
                    om = O.OracleMesh(m.arrays())
                    ref = O.OracleHierarchy(om).transport_step(
                        0.0, 4e7, inputs[0].dt, inp.t0, inp.source, tol=1e-13,
                        edge_g=om.directed_conductance(inp.edge_conductance))
                    assert np.max(np.abs(got - ref["t_new"])) <= 2e-6
    # the plain V-cycle again: the scale is part of the settings, not left behind
    t["coarse_correction"] = 1.0
    batch.set_tuning(t)
    assert batch.tuning["coarse_correction"] == 1.0
