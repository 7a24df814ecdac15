"""CUDA-graph replay and explicit launch shapes of the mixed form (C ABI)."""

import numpy as np
import pytest

from mpmc_hnu_gb300 import synth


def _device_solve(torch, g, p, t, z, bufs=None):
    n = g.n
    ncell = p.shape[0]
    if bufs is None:
        from mpmc_hnu_gb300 import flash

        rows = flash.output_rows(n)
        dtypes = {f: d for f, d, _ in flash.OUTPUT_FIELDS}
        bufs = {"p": torch.empty(ncell, dtype=torch.float64, device="cuda"),
                "t": torch.empty(ncell, dtype=torch.float64, device="cuda"),
                "z": torch.empty((n, ncell), dtype=torch.float64, device="cuda"),
                "out": {f: torch.empty((rows[f], ncell), device="cuda",
                                       dtype=torch.int32 if dtypes[f] == np.int32 else torch.float64)
                        for f in g.fields()}}
    bufs["p"].copy_(torch.from_numpy(p))
    bufs["t"].copy_(torch.from_numpy(t))
    bufs["z"].copy_(torch.from_numpy(np.ascontiguousarray(z)))
    torch.cuda.synchronize()
    g.solve_device(ncell, bufs["p"].data_ptr(), bufs["t"].data_ptr(), bufs["z"].data_ptr(),
                   {f: v.data_ptr() for f, v in bufs["out"].items()}, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return {f: v.cpu().numpy() for f, v in bufs["out"].items()}, bufs


@pytest.mark.gpu
def test_graph_replay_matches_direct_launches(gpu_lib):
    import torch

    n = 8
    mix = synth.make_mixture(n, 41)
    plain = gpu_lib.GpuFlash(mix, form="mixed", sensitivity=True)
    graphed = gpu_lib.GpuFlash(mix, form="mixed", sensitivity=True, graphs=True)
    a = synth.make_cells(n, 640, 41)
    b = synth.make_cells(n, 640, 42)
    want_a, _ = _device_solve(torch, plain, *a)
    want_b, _ = _device_solve(torch, plain, *b)
    got_a, bufs = _device_solve(torch, graphed, *a)          # capture
    got_b, _ = _device_solve(torch, graphed, *b, bufs=bufs)  # replay on new contents, same buffers
    got_a2, _ = _device_solve(torch, graphed, *a, bufs=bufs)
    for want, got in ((want_a, got_a), (want_b, got_b), (want_a, got_a2)):
        for f in want:
            np.testing.assert_array_equal(want[f], got[f], err_msg=f)
    plain.close()
    graphed.close()


@pytest.mark.gpu
def test_launch_shapes_keep_the_results(gpu_lib, oracle_lib):
    from tests import parity

    n = 10
    mix = synth.make_mixture(n, 43)
    p, t, z = synth.make_cells(n, 512, 43)
    ref = oracle_lib.flash(mix, p, t, z, threads=8)
    g = gpu_lib.GpuFlash(mix, form="mixed")
    # residency and item forms (the SS -> Newton switch moves rounding of the
    # FP32 stopping point and is guarded by the autotuner instead)
    for shape in ([0] * 7, [2, 2, 1, 4, 8, 8], [4, 4, 4, 1, 4, 0], [0, 0, 0, 0, 0, 15], [0, 0, 0, 0, 0, 32 + 128],
                  [0, 0, 0, 0, 0, 64, 0, 2], [0] * 8 + [128, 64]):
        g.set_launch_shape(shape)
        out = g.solve(p, t, z)
        rep = parity.flash_report(out, ref, mix, p, t, z)
        parity.assert_flash_parity(rep)
    with pytest.raises(gpu_lib.FlashError):
        g.set_launch_shape([0] * 11)
    with pytest.raises(gpu_lib.FlashError):
        g.set_launch_shape([0] * 8 + [513])
    g.close()
