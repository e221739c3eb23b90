"""GB300-native (sm_103a) implicit heat-transport sub-step of PlanetSim.

The product is the C-ABI library ``lib/libplanetsim_gb300.so`` (declared in
``include/planetsim_gb300.h``); this package builds it in-tree and mirrors the
reference's C++ operator and solver API over it.
"""
from .api import (  # noqa: F401
    Batch,
    GraphMultigrid,
    LaneBatch,
    default_lanes,
    PlanetMesh,
    QuarticResponse,
    TransportGraph,
    TunedSolo,
    agglomerated_transport_graph,
    column_constants,
    column_radiation,
    diffusion_source,
    divergence,
    gradient,
    group_mean,
    group_scatter,
    laplacian,
    make_icosphere,
    quartic_response,
    mesh_transport_graph,
    solve_implicit_transport,
    solve_newton_system,
    solve_options,
    transport_settings,
    transport_step,
    transport_step_multi,
)
from .capi import GB300Error  # noqa: F401
from .nonsym import (  # noqa: F401
    AdvectionDiffusion,
    IncompleteLU,
    advection_diffusion_source,
    solve_implicit_advection_diffusion,
    solve_implicit_tracer,
)
