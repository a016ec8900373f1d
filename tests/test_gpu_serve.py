"""The serving loop (continuous batching of offscreen clients over several
queues): every request completes, requests overlap on the device, each
client's image is the same rendered in the mix as rendered alone (and as the
oracle's), and clients beyond the HBM budget are served by evicting idle
ones."""
import numpy as np
import pytest

import cpvulkan_gb300 as c
from tests.parity import compare

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def served(gpu_ctx):
    server = c.Server(gpu_ctx, clients=12, slots=8, mean_interarrival_ms=1.0, duration_s=0.6, seed=9, min_tris=1000,
                      max_tris=60000, max_side=512)
    stats = server.run()
    yield server, stats
    server.close()


def test_every_request_completes(served):
    server, st = served
    assert st["resident_clients"] == 12
    assert st["requests"] > 100 and st["completed"] == st["requests"]
    assert st["triangles"] > 0 and st["mtri_s"] > 0
    assert st["max_in_flight"] > 1  # requests overlapped
    assert 0 < st["submit_p50_ms"] <= st["submit_p99_ms"]
    assert st["latency_p50_ms"] >= st["queue_p50_ms"]


def test_mixed_equals_alone(served, oracle):
    server, _ = served
    for i in range(server.clients):
        view = server.client(i)
        mixed = view.readback()  # the client's last request in the mix
        view.render(1)           # alone: nothing else in flight
        alone = view.readback()
        assert np.array_equal(mixed[0], alone[0]), i
        assert np.array_equal(mixed[1], alone[1]), i
        if i < 3:
            ocol, odep, _ = oracle.render(view.scene)
            report = compare(view.scene, alone[0], alone[1], ocol, odep)
            assert report["color_pixels_differing"] == 0, report


def test_budget_limits_residency(gpu_ctx):
    # A budget for about two small clients and no admission on demand: the
    # rest stay non-resident and their requests are not generated.
    server = c.Server(gpu_ctx, clients=6, slots=4, mean_interarrival_ms=2.0, duration_s=0.2, seed=3, hbm_budget_bytes=6 << 20,
                      min_tris=1000, max_tris=2000, max_side=256, admit_on_demand=False)
    try:
        st = server.run()
        assert 0 < st["resident_clients"] < 6
        assert st["resident_bytes"] <= 6 << 20
        assert st["completed"] == st["requests"]
        assert sum(server.client(i) is None for i in range(6)) == 6 - st["resident_clients"]
    finally:
        server.close()


def test_eviction_admits_on_demand(gpu_ctx, oracle):
    # A budget for about three of eight clients: every client's requests are
    # served, by making it resident when its request is admitted and
    # evicting idle clients, least recently used first.
    server = c.Server(gpu_ctx, clients=8, slots=4, mean_interarrival_ms=4.0, duration_s=0.4, seed=4, hbm_budget_bytes=10 << 20,
                      min_tris=1000, max_tris=20000, max_side=256)
    try:
        st = server.run()
        assert st["requests"] > 50 and st["completed"] == st["requests"]
        assert st["residencies"] > 0 and st["evictions"] > 0
        assert st["resident_bytes"] <= 10 << 20
        assert 0 < st["residency_p50_ms"] <= st["residency_p99_ms"]
        checked = 0
        for i in range(server.clients):
            view = server.client(i)
            if view is None:
                continue
            mixed = view.readback()  # its last request, possibly after being made resident again
            view.render(1)
            alone = view.readback()
            assert np.array_equal(mixed[0], alone[0]), i
            ocol, odep, _ = oracle.render(view.scene)
            report = compare(view.scene, alone[0], alone[1], ocol, odep)
            assert report["color_pixels_differing"] == 0, report
            checked += 1
        assert checked == st["resident_clients"] > 0
    finally:
        server.close()
