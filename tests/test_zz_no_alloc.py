"""The no-allocation entry point against the allocating one (through the C ABI).

Collected last on purpose: it must give the same results in a fresh process
and after every other test has used the device.
"""

import numpy as np
import pytest

from mpmc_hnu_gb300 import synth

# results come from the same kernels on the same inputs: they agree to rounding
# of nothing at all, so the tolerance only guards against a flaky comparison
RTOL, ATOL = 1e-12, 1e-14


def _device_buffers(torch, g, ncell):
    rows = {f: r(g.n) for f, _, r in g_fields()}
    dtypes = {f: d for f, d, _ in g_fields()}
    out = {}
    for f in g.fields():
        tdt = torch.int32 if dtypes[f] == np.int32 else torch.float64
        out[f] = torch.full((rows[f], ncell), -7, dtype=tdt, device="cuda")
    return out


def g_fields():
    from mpmc_hnu_gb300 import flash

    return flash.OUTPUT_FIELDS


def _run(torch, g, p, t, z, noalloc):
    ncell = p.shape[0]
    dp = torch.from_numpy(p).cuda()
    dt = torch.from_numpy(t).cuda()
    dz = torch.from_numpy(np.ascontiguousarray(z)).cuda()
    out = _device_buffers(torch, g, ncell)
    ptrs = {f: v.data_ptr() for f, v in out.items()}
    stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    call = g.solve_device_noalloc if noalloc else g.solve_device
    call(ncell, dp.data_ptr(), dt.data_ptr(), dz.data_ptr(), ptrs, stream)
    torch.cuda.synchronize()
    return {f: v.cpu().numpy() for f, v in out.items()}


def _assert_same(a, b):
    for f in a:
        if a[f].dtype == np.int32:
            np.testing.assert_array_equal(a[f], b[f], err_msg=f)
        else:
            np.testing.assert_allclose(a[f], b[f], rtol=RTOL, atol=ATOL, equal_nan=True, err_msg=f)


@pytest.mark.gpu
@pytest.mark.parametrize("n,sensitivity", [(6, True), (10, False)])
def test_noalloc_matches_solve_device_twice(gpu_lib, n, sensitivity):
    import torch

    mix = synth.make_mixture(n, 11)
    g = gpu_lib.GpuFlash(mix, form="mixed", sensitivity=sensitivity)
    batches = [synth.make_cells(n, 512, 11), synth.make_cells(n, 300, 12, offset=7000)]
    # two no-allocation calls in a row, each against the allocating entry point
    for p, t, z in batches:
        got = _run(torch, g, p, t, z, noalloc=True)
        want = _run(torch, g, p, t, z, noalloc=False)
        assert (got["status"] == 1).any()
        _assert_same(got, want)
    # and the same batch again, back to back, with the scratch already used
    p, t, z = batches[0]
    first = _run(torch, g, p, t, z, noalloc=True)
    again = _run(torch, g, p, t, z, noalloc=True)
    _assert_same(first, again)
    g.close()


@pytest.mark.gpu
def test_noalloc_rejects_what_it_cannot_hold(gpu_lib):
    import torch

    n = 20
    mix = synth.make_mixture(n, 4)
    g = gpu_lib.GpuFlash(mix, form="mixed")
    ncell = 8192  # needs about 80 MiB of work buffers at 20 components
    p, t, z = synth.make_cells(n, ncell, 4)
    dp = torch.from_numpy(p).cuda()
    dt = torch.from_numpy(t).cuda()
    dz = torch.from_numpy(z).cuda()
    status = torch.empty(ncell, dtype=torch.int32, device="cuda")
    with pytest.raises(gpu_lib.FlashError) as err:
        g.solve_device_noalloc(ncell, dp.data_ptr(), dt.data_ptr(), dz.data_ptr(), {"status": status.data_ptr()})
    assert err.value.code == 1 and "bytes of scratch" in str(err.value)
    g.close()
    plain = gpu_lib.GpuFlash(mix, form="plain")
    with pytest.raises(gpu_lib.FlashError) as err:
        plain.solve_device_noalloc(ncell, dp.data_ptr(), dt.data_ptr(), dz.data_ptr(), {"status": status.data_ptr()})
    assert err.value.code == 4
    plain.close()
