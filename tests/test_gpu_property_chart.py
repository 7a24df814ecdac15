"""Selected-phase property chart on the GPU (mpmc_gpu_flash_property_chart)
against the recorded reference outputs (tests/golden/property_chart_reference.npz)
and against the oracle on larger seeded charts.

Statuses must be identical; values agree within 1e-10 relative and Jacobian
entries within 1e-9 of their row's largest column-scaled derivative
(tests/chart_parity.py).  Failed cells are NaN everywhere.
"""

import numpy as np
import pytest

from mpmc_hnu_gb300 import synth
from mpmc_hnu_gb300.flash import chart_shape
from tests import chart_cases
from tests.chart_parity import check_chart
from tests.test_oracle_property_chart import golden_cases


def _oracle(lib, mix, spec, q, dep):
    return lib.property_chart(mix, spec.phases, spec.root_index, spec.molar_mass, spec.viscosity, spec.enthalpy, q,
                              dep)


@pytest.mark.gpu
def test_chart_matches_recorded_reference(gpu_lib):
    for name, mix, spec, q, dep, ref in golden_cases():
        g = gpu_lib.GpuFlash(mix, form="plain")
        out = g.property_chart(spec, q, dep)
        g.close()
        check_chart(out, ref, q, name)


@pytest.mark.gpu
@pytest.mark.parametrize("n,phases,roots,ncell", [(2, 2, [0, 0], 4096), (4, 1, [0], 4096), (10, 2, [0, 0], 20000),
                                                  (10, 3, [0, 1, 2], 8192), (12, 3, [0, 0, 0], 8192),
                                                  (20, 2, [0, 0], 4096)])
def test_chart_matches_oracle(gpu_lib, oracle_lib, n, phases, roots, ncell):
    name, mix, spec, q, dep = chart_cases.random_case("gpu", n, phases, roots, ncell, 700 + n)
    g = gpu_lib.GpuFlash(mix, form="mixed")
    out = g.property_chart(spec, q, dep)
    g.close()
    ref = _oracle(oracle_lib, mix, spec, q, dep)
    check_chart(out, ref, q, f"n{n} P{phases}")


@pytest.mark.gpu
def test_chart_device_entry_and_default_pivot(gpu_lib, oracle_lib):
    """The device-buffer entry on a torch stream equals the host entry; a null
    pivot array means the last component of every phase; values alone can be
    requested."""
    import torch

    n, phases = 10, 2
    ncell = 5000
    mix = synth.make_mixture(n, 1011)
    spec = chart_cases.random_spec(n, phases, [0, 0], 77)
    last = np.full((phases, ncell), n - 1, np.int32)
    # any drawn state is a valid chart for the last component as the pivot:
    # its independent entries are positive with a sum below one
    q_last, _ = chart_cases.random_states(n, phases, ncell, 78)
    g = gpu_lib.GpuFlash(mix, form="mixed")
    host = g.property_chart(spec, q_last, None)
    explicit = g.property_chart(spec, q_last, last)
    values_only = g.property_chart(spec, q_last, None, jacobian=False)
    rows, cols = chart_shape(n, phases)
    dev = torch.device("cuda:0")
    dq = torch.from_numpy(np.ascontiguousarray(q_last)).to(dev).contiguous()
    st = torch.empty(ncell, dtype=torch.int32, device=dev)
    vals = torch.empty((rows, ncell), dtype=torch.float64, device=dev)
    jac = torch.empty((rows, cols, ncell), dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(device=dev)
    stream.wait_stream(torch.cuda.current_stream(dev))  # the input copy and allocations
    with torch.cuda.stream(stream):
        g.property_chart_device(spec, ncell, dq.data_ptr(), 0,
                                {"status": st.data_ptr(), "values": vals.data_ptr(), "jacobian": jac.data_ptr()},
                                stream=stream.cuda_stream)
    stream.synchronize()
    g.close()
    for k in ("status", "values", "jacobian"):
        assert np.array_equal(host[k], explicit[k], equal_nan=True), k
    assert np.array_equal(values_only["values"], host["values"], equal_nan=True)
    assert np.array_equal(st.cpu().numpy(), host["status"])
    assert np.array_equal(vals.cpu().numpy(), host["values"], equal_nan=True)
    assert np.array_equal(jac.cpu().numpy(), host["jacobian"], equal_nan=True)
    check_chart(host, _oracle(oracle_lib, mix, spec, q_last, None), q_last, "default pivot")
