"""The serving loop's admission by HBM budget (host logic, no GPU): lanes are built while
their bytes fit, the least recently used idle lane is evicted first, busy lanes and lanes
with queued requests are never evicted, and a request waits (None) when nothing can go."""
from types import SimpleNamespace

import pytest


@pytest.fixture
def server(monkeypatch):
    import torch

    from planet_game_gb300 import serve

    built = []

    class FakeBatch:
        def __init__(self, meshes):
            built.append(len(meshes))

        def set_edge_conductance(self, edges):
            pass

        def set_tuning(self, tuning):
            pass

    monkeypatch.setattr(serve.api, "Batch", FakeBatch)
    monkeypatch.setattr(torch.cuda, "Stream", lambda *a, **k: None)

    def planets(level, cells):
        return [serve.PlanetState(level, 6.371e6, SimpleNamespace(cell_count=cells), None, None, 4e7, 1.0, 1.0)
                for _ in range(2)]

    # lane bytes = cells x 700: L4 1.4 MB, L5 5.6 MB, L6 22.4 MB
    pop = {4: planets(4, 1000), 5: planets(5, 4000), 6: planets(6, 16000)}
    srv = serve.Server(pop, budget_bytes=25e6, autotune=False, device=torch.device("cpu"))
    yield srv, built
    srv.close()


def test_lanes_fit_then_the_least_recently_used_idle_lane_goes(server):
    srv, built = server
    with srv.lock:
        l4, l5 = srv._admit(4), srv._admit(5)
    assert l4 is not None and l5 is not None and srv.resident_bytes == 7_000_000
    l4.last_used, l5.last_used = 1.0, 2.0
    with srv.lock:
        l6 = srv._admit(6)          # 7.0 + 22.4 > 25: both idle lanes go, oldest first
    assert l6 is not None and srv.evictions == 2 and srv.resident_bytes == 22_400_000
    assert l4.batch is None and l5.batch is None and built == [2, 2, 2]


def test_busy_or_queued_lanes_stay_and_requests_wait(server):
    srv, _ = server
    with srv.lock:
        l6 = srv._admit(6)
        l6.busy = True              # a round is running on it
        l4 = srv._admit(4)          # 22.4 + 1.4 fits
        assert l4 is not None
        l4.pending[0].append(object())   # a queued request keeps the lane
        assert srv._admit(5) is None     # 23.8 + 5.6 > 25 and nothing can be evicted
        assert srv.evictions == 0
        l4.pending[0].clear()
        l4.last_used = 1.0
        assert srv._admit(5) is None     # l4 goes, but 22.4 + 5.6 still exceeds the budget
        assert srv.evictions == 1 and l4.batch is None
        l6.busy = False
        l6.last_used = 2.0
        assert srv._admit(5) is not None  # now l6 can go too
        assert srv.resident_bytes == 5_600_000
