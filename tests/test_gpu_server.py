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
