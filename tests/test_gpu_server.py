"""The continuous-batching flash server (through the C ABI).

A request's result must be the same alone and in a mix with other requests
(same and other mixtures, batched into one launch or overlapping on other
streams).  Every cell is computed from its own inputs only, so the bar is
bit-identical; it is also checked against the single-handle entry point.
"""

import threading

import numpy as np
import pytest

from mpmc_hnu_gb300 import synth


def _same(a, b):
    for f in a:
        np.testing.assert_array_equal(np.asarray(a[f]), np.asarray(b[f]), err_msg=f)


@pytest.mark.gpu
def test_request_alone_equals_request_in_the_mix(gpu_lib):
    mix_a = synth.make_mixture(6, 21)
    mix_b = synth.make_mixture(10, 22)
    server = gpu_lib.FlashServer(slots=3, max_batch_cells=8192, memory_budget_bytes=8 << 30)
    ida, idb = server.add_mixture(mix_a), server.add_mixture(mix_b)
    p, t, z = synth.make_cells(6, 700, 21)

    alone, _ = server.wait(server.submit(ida, p, t, z))

    # the same request in the middle of a burst of same- and other-mixture requests
    tickets = []
    for k in range(12):
        mid, n = (ida, 6) if k % 2 == 0 else (idb, 10)
        q = synth.make_cells(n, 50 + 97 * k, 100 + k)
        tickets.append(server.submit(mid, *q))
        if k == 5:
            target = server.submit(ida, p, t, z)
    in_mix, _ = server.wait(target)
    for tk in tickets:
        server.wait(tk)
    st = server.stats()
    server.close()
    _same(alone, in_mix)
    assert st["most_requests_in_batch"] > 1, st

    # and the same as the single-handle entry point on the same cells
    g = gpu_lib.GpuFlash(mix_a, form="mixed")
    direct = g.solve(p, t, z)
    g.close()
    _same(alone, {f: direct[f] for f in alone})


@pytest.mark.gpu
def test_concurrent_clients_all_complete(gpu_lib):
    mixes = [synth.make_mixture(n, 30 + n) for n in (3, 6, 10, 20)]
    server = gpu_lib.FlashServer(slots=4, max_batch_cells=16384, memory_budget_bytes=16 << 30)
    ids = [server.add_mixture(m) for m in mixes]
    results = {}
    errors = []

    def client(c):
        try:
            rng = np.random.default_rng(c)
            for k in range(6):
                j = int(rng.integers(0, 4))
                n = mixes[j].n
                ncell = int(np.exp(rng.uniform(0, np.log(4096))))
                q = synth.make_cells(n, ncell, 1000 * c + k)
                out, lat = server.wait(server.submit(ids[j], *q))
                results[(c, k)] = (j, q, out, lat)
        except Exception as exc:  # pragma: no cover - reported below
            errors.append(exc)

    threads = [threading.Thread(target=client, args=(c,)) for c in range(6)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    st = server.stats()
    server.close()
    assert not errors, errors
    assert len(results) == 36 and st["completed"] == 36, st
    # spot-check a few against the single-handle entry point
    for key in list(results)[:6]:
        j, q, out, lat = results[key]
        g = gpu_lib.GpuFlash(mixes[j], form="mixed")
        direct = g.solve(*q)
        g.close()
        _same(out, {f: direct[f] for f in out})
        assert lat > 0.0


@pytest.mark.gpu
def test_server_rejects_what_it_cannot_serve(gpu_lib):
    server = gpu_lib.FlashServer(slots=1, max_batch_cells=1024, memory_budget_bytes=2 << 30)
    mid = server.add_mixture(synth.make_mixture(4, 3))
    p, t, z = synth.make_cells(4, 2048, 3)
    with pytest.raises(gpu_lib.FlashError) as err:
        server.submit(mid, p, t, z)
    assert err.value.code == 1
    with pytest.raises(gpu_lib.FlashError) as err:
        server.submit(mid, p[:8], t[:8], z[:, :8], fields=["status", "d_ln_k"])
    assert err.value.code == 4
    with pytest.raises(gpu_lib.FlashError):
        gpu_lib.FlashServer(slots=1, max_batch_cells=1 << 20, memory_budget_bytes=1 << 20)
    server.close()


@pytest.mark.gpu
def test_latency_slots_and_chunking_keep_every_result(gpu_lib):
    """Small requests on a latency slot, large ones cut into chunks that
    interleave on the other slots: every request equals the single-handle
    solve bit for bit (counters included)."""
    mixes = [synth.make_mixture(n, 60 + n) for n in (6, 10)]
    server = gpu_lib.FlashServer(slots=3, max_batch_cells=4096, memory_budget_bytes=8 << 30,
                                 policy={"small_request_cells": 512, "latency_slots": 1, "latency_batch_cells": 1024,
                                         "chunk_cells": 1024, "max_request_cells": 16384})
    ids = [server.add_mixture(m) for m in mixes]
    reqs = []
    for k, ncell in enumerate([5000, 300, 2100, 40, 512, 9000, 1, 777]):
        j = k % 2
        q = synth.make_cells(mixes[j].n, ncell, 500 + k)
        reqs.append((j, q, server.submit(ids[j], *q)))
    outs = [(j, q, server.wait(tk)[0]) for j, q, tk in reqs]
    st = server.stats()
    server.close()
    assert st["completed"] == len(reqs) and st["batches"] > len(reqs)  # the large ones were chunked
    for j, q, out in outs:
        g = gpu_lib.GpuFlash(mixes[j], form="mixed")
        direct = g.solve(*q)
        g.close()
        _same(out, {f: direct[f] for f in out})


@pytest.mark.gpu
def test_deadline_drops_a_request_without_touching_the_others(gpu_lib):
    """One slot busy with a large request: a small request whose deadline
    passes while it waits is dropped (MPMC_ERR_DEADLINE), its outputs are not
    written, and the large request's results are unaffected."""
    mix = synth.make_mixture(20, 71)
    server = gpu_lib.FlashServer(slots=1, max_batch_cells=32768, memory_budget_bytes=16 << 30)
    mid = server.add_mixture(mix)
    big = synth.make_cells(20, 32768, 72)
    small = synth.make_cells(20, 16, 73)
    tb = server.submit(mid, *big)
    ts = server.submit(mid, *small, deadline_s=1e-3)
    with pytest.raises(gpu_lib.FlashError) as err:
        server.wait(ts)
    assert err.value.code == gpu_lib.ERR_DEADLINE
    out, _ = server.wait(tb)
    st = server.stats()
    # a deadline must be positive
    with pytest.raises(gpu_lib.FlashError):
        server.submit(mid, *small, deadline_s=-1.0)
    server.close()
    assert st["expired"] == 1 and st["completed"] == 2
    g = gpu_lib.GpuFlash(mix, form="mixed")
    direct = g.solve(*big)
    g.close()
    _same(out, {f: direct[f] for f in out})


@pytest.mark.gpu
def test_concurrency_limit_refuses_at_once(gpu_lib):
    """With max_in_flight = 2 a third submit fails at once with MPMC_ERR_BUSY
    (nothing is queued), and succeeds again once a request completed."""
    mix = synth.make_mixture(10, 81)
    server = gpu_lib.FlashServer(slots=1, max_batch_cells=16384, memory_budget_bytes=8 << 30,
                                 policy={"max_in_flight": 2})
    mid = server.add_mixture(mix)
    a = synth.make_cells(10, 16384, 82)
    b = synth.make_cells(10, 100, 83)
    ta, tb = server.submit(mid, *a), server.submit(mid, *b)
    with pytest.raises(gpu_lib.FlashError) as err:
        server.submit(mid, *b)
    assert err.value.code == gpu_lib.ERR_BUSY
    server.wait(ta)
    server.wait(tb)
    tc = server.submit(mid, *b)
    out, _ = server.wait(tc)
    st = server.stats()
    server.close()
    assert st["refused_busy"] == 1 and st["completed"] == 3
    assert out["status"].shape == (100,)


@pytest.mark.gpu
def test_warm_cache_reuses_ln_k_of_earlier_requests(gpu_lib):
    """A request that re-queries an earlier request's compositions at nearby
    (p, T) starts those cells from the cached ln K on the device: its statuses
    equal the cold solve's and its two-phase pairs agree to 1e-8."""
    mix = synth.make_mixture(6, 91)
    server = gpu_lib.FlashServer(slots=2, max_batch_cells=8192, memory_budget_bytes=8 << 30, warm_cache=True)
    mid = server.add_mixture(mix)
    p, t, z = synth.make_cells(6, 4000, 92)
    server.wait(server.submit(mid, p, t, z))
    rng = np.random.default_rng(93)
    p2 = p * np.exp(rng.normal(0.0, 0.02, p.size))
    t2 = t + rng.normal(0.0, 1.0, t.size)
    out, _ = server.wait(server.submit(mid, p2, t2, z))
    st = server.stats()
    server.close()
    g = gpu_lib.GpuFlash(mix, form="mixed")
    cold = g.solve(p2, t2, z)
    g.close()
    assert st["warm_cells"] > 100, st
    np.testing.assert_array_equal(out["status"], cold["status"])
    two = cold["status"] == 1
    assert np.abs(out["ln_k"][:, two] - cold["ln_k"][:, two]).max() <= 1e-8
