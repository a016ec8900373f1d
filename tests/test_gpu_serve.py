"""The serving loop (continuous batching of resident offscreen clients over
several queues): every request completes, requests overlap on the device,
and each client's image is the same rendered in the mix as rendered alone
(and as the oracle's)."""
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
    # A budget for about two small clients: the rest stay non-resident and
    # their requests are not generated.
    server = c.Server(gpu_ctx, clients=6, slots=4, mean_interarrival_ms=2.0, duration_s=0.2, seed=3, hbm_budget_bytes=6 << 20,
                      min_tris=1000, max_tris=2000, max_side=256)
    try:
        st = server.run()
        assert 0 < st["resident_clients"] < 6
        assert st["resident_bytes"] <= 6 << 20
        assert st["completed"] == st["requests"]
        assert sum(server.client(i) is None for i in range(6)) == 6 - st["resident_clients"]
    finally:
        server.close()
