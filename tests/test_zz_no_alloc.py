"""GPU test of the allocation-free probability entry point
(qg_calc_probability_noalloc in include/qgate_gb300.h).

That entry point exists for callers that cannot let the library allocate
device memory (an application that owns all of it in its own pool, or a loop
that must not take the synchronisation of a cudaMalloc): they pass their own
device buffers and the reduction's scratch comes from a fixed device array.
This file is named so that pytest collects it last; it also passes alone in a
fresh process.  It calls the entry point through the C ABI on device memory
owned by the test (torch tensors), twice in a row, and compares each result
with the regular entry point qg_qubit_processor_calc_probability on the same
state, at the tolerance the other probability tests use (1e-12 for
complex128, 2e-6 for complex64 amplitudes accumulated in FP64)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('dtype', [np.float64, np.float32], ids=['c128', 'c64'])
def test_noalloc_probability_matches_regular_entry_point(rt, dtype):
    import torch
    from qgate_gb300 import _native as nat
    from tests.gpu_helpers import apply_ops, new_state, random_ops

    n = 14
    rng = np.random.default_rng(21)
    qs = new_state(rt, n, dtype)
    apply_ops(qs, random_ops(rng, n, 60))
    raw = qs.get_raw()
    tdtype = torch.complex128 if dtype == np.float64 else torch.complex64
    state = torch.from_numpy(raw).to(device='cuda', dtype=tdtype)
    out = torch.full((2,), -1.0, dtype=torch.float64, device='cuda')
    prec = nat.PREC_FP64 if dtype == np.float64 else nat.PREC_FP32
    stream = torch.cuda.current_stream().cuda_stream
    tol = 1e-12 if dtype == np.float64 else 2e-6
    for lanes in ((3, 11), (0, n - 1)):
        for i, lane in enumerate(lanes):  # two calls in a row
            nat.call('qg_calc_probability_noalloc', prec, state.data_ptr(), n, lane,
                     out.data_ptr() + 8 * i, stream)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        for i, lane in enumerate(lanes):
            want = qs.processor.calc_probability(qs, lane)
            assert abs(got[i] - want) < tol, (lane, got[i], want)


def test_noalloc_rejects_out_of_range_sizes(rt):
    from qgate_gb300 import _native as nat
    with pytest.raises(ValueError, match='n_lanes'):
        nat.call('qg_calc_probability_noalloc', nat.PREC_FP32, 16, 41, 0, 16, 0)
    with pytest.raises(ValueError, match='local_lane'):
        nat.call('qg_calc_probability_noalloc', nat.PREC_FP32, 16, 4, 4, 16, 0)


def test_noalloc_rejects_misaligned_pointers(rt):
    """A complex64 state that starts 8 bytes into a buffer (a slice from the
    second amplitude) is refused on the host before any launch, as is an
    output pointer that is not 8-byte aligned; nothing runs on the GPU."""
    import torch
    from qgate_gb300 import _native as nat
    state = torch.zeros(1 << 6, dtype=torch.complex64, device='cuda')
    out = torch.zeros(2, dtype=torch.float64, device='cuda')
    with pytest.raises(ValueError, match='16-byte aligned'):
        nat.call('qg_calc_probability_noalloc', nat.PREC_FP32, state.data_ptr() + 8, 5, 0,
                 out.data_ptr(), 0)
    with pytest.raises(ValueError, match='8-byte aligned'):
        nat.call('qg_calc_probability_noalloc', nat.PREC_FP32, state.data_ptr(), 5, 0,
                 out.data_ptr() + 4, 0)
