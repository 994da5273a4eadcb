"""The serving loop on the GPU: requests overlap on the device (several
slots), and each result is identical alone, in the mix, and to a direct
cor_trace_batch of its scans."""
from __future__ import annotations

import numpy as np
import pytest

import cortrace as ct
import serve

pytestmark = pytest.mark.gpu


def _small(reqs):
    for r in reqs:
        r.rig = (1.0, 20.0, 1.0)          # 20 rigidities per site-direction
    return reqs


def test_gpu_serving_results_alone_and_in_mix(ctx):
    mix = _small(serve.poisson_stream(21, 50.0, 8, max_box_sites=4))
    out = serve.run_stream(serve.Server(0, slots=3), mix)
    print("serving (small requests):", out)
    assert out["completed"] == 8 and out["batches"] >= 1
    alone = _small([serve.poisson_stream(21, 50.0, 8, max_box_sites=4)[2]])
    alone[0].arrival = 0.0
    serve.run_stream(serve.Server(0, slots=1), alone)
    assert np.array_equal(alone[0].result.view(np.uint8), mix[2].result.view(np.uint8))
    for r in mix[:3]:
        p = ct.internal_setup("igrf14", r.time7, parmod=r.parmod)
        direct = ctx.trace_batch(serve.request_jobs(r, 0), p, models=ct.model_set(ct.INTERNAL_SH, r.external))
        assert np.array_equal(direct.sites.view(np.uint8), r.result.view(np.uint8))


def test_stream_server_alone_and_in_mix(ctx):
    """The stream-backed server: requests in flight together on one resident
    kernel give each request the bytes it gets alone; with IGRF-14 only, also
    the bytes of a direct cor_trace_batch of its scans."""
    mix = _small(serve.poisson_stream(25, 50.0, 8, max_box_sites=4))
    for r in mix:
        r.external = ct.EXTERNAL_NONE
    out = serve.run_stream(serve.StreamServer(0, externals=(ct.EXTERNAL_NONE,)), mix)
    print("stream serving (small requests):", out)
    assert out["completed"] == 8 and out["rejected"] == 0
    alone = _small([serve.poisson_stream(25, 50.0, 8, max_box_sites=4)[3]])
    alone[0].external = ct.EXTERNAL_NONE
    alone[0].arrival = 0.0
    serve.run_stream(serve.StreamServer(0, externals=(ct.EXTERNAL_NONE,)), alone)
    assert np.array_equal(alone[0].result.view(np.uint8), mix[3].result.view(np.uint8))
    for r in mix[:4]:
        p = ct.internal_setup("igrf14", r.time7, parmod=r.parmod)
        direct = ctx.trace_batch(serve.request_jobs(r, 0), p, models=ct.model_set(ct.INTERNAL_SH))
        assert np.array_equal(direct.sites.view(np.uint8), r.result.view(np.uint8))


def test_stream_server_t96_alone_and_in_mix():
    mix = _small(serve.poisson_stream(27, 50.0, 6, ct.EXTERNAL_T96, max_box_sites=4))
    out = serve.run_stream(serve.StreamServer(0, externals=(ct.EXTERNAL_T96,)), mix)
    assert out["completed"] == 6
    alone = _small([serve.poisson_stream(27, 50.0, 6, ct.EXTERNAL_T96, max_box_sites=4)[1]])
    alone[0].arrival = 0.0
    serve.run_stream(serve.StreamServer(0, externals=(ct.EXTERNAL_T96,)), alone)
    assert np.array_equal(alone[0].result.view(np.uint8), mix[1].result.view(np.uint8))
