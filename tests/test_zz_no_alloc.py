"""GPU test of qvmg_sample_noalloc, the sampling entry point that allocates
nothing.

It exists for callers that cannot allocate device memory themselves (a host
that owns the device pool and only lends out slices of it, or a loop that
cannot pay for cudaMalloc's synchronisation), so they cannot create a state
handle.  Here the test plays such a caller: it holds the amplitudes, draws and
output in device buffers it owns (allocated by torch, as a host framework
would) and calls the entry point through the C ABI.  Its indices must equal
those of the allocating entry point, qvmg_sample, on the same amplitudes and
draws -- exactly, as for every integer result in these tests -- on two calls
in a row, since all calls share the one fixed scratch array.

This file is named to be collected last, so a run that stops at the first
failure has run every other test before it.
"""
import numpy as np
import pytest

from qvm_gb300 import CudaPureState, circuits
from qvm_gb300 import _lib as L

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_noalloc_sampling_matches_allocating_sampler(gpu, prec):
    import torch

    n = 16
    wf = circuits.random_state(n, seed=21)
    ref = CudaPureState(n, prec)
    ref.set_state_elements(wf)
    if prec == "fp64":
        amps = torch.from_numpy(wf.view(np.float64).copy()).cuda()
    else:
        amps = torch.from_numpy(wf.astype(np.complex64).view(np.float32).copy()).cuda()
    stream = torch.cuda.current_stream()
    for call in range(2):
        draws = np.random.default_rng(100 + call).random(1000)
        d_draws = torch.from_numpy(draws).cuda()
        for rule, name in ((L.SAMPLE_BISECT, "bisect"), (L.SAMPLE_CDF, "cdf")):
            d_out = torch.full((len(draws),), -1, dtype=torch.int64, device="cuda")
            L.check(L.lib().qvmg_sample_noalloc(amps.data_ptr(), n, ref.precision,
                                                d_draws.data_ptr(), len(draws), rule,
                                                d_out.data_ptr(), stream.cuda_stream))
            stream.synchronize()
            got = d_out.cpu().numpy().astype(np.uint64)
            want = ref.sample(draws, rule=name)
            np.testing.assert_array_equal(got, want)
    ref.free()


def test_noalloc_at_its_30_qubit_limit(gpu):
    """At 30 qubits the block sums fill the fixed array exactly (2^18 blocks
    plus the total).  FP32 amplitudes made on the device, 300 draws of which
    some sit at and near 1.0, on two calls in a row: identical to
    qvmg_sample."""
    import torch

    n = 30
    gen = torch.Generator(device="cuda").manual_seed(30)
    amps = torch.randn(2 << n, dtype=torch.float32, device="cuda", generator=gen)
    amps *= float(1.0 / torch.linalg.vector_norm(amps.double()).item())
    ref = CudaPureState(n, "fp32")
    ref.set_state_elements(amps.cpu().numpy().view(np.complex64).astype(np.complex128))
    stream = torch.cuda.current_stream()
    edge = np.array([0.0, 1e-12, 0.5, 1 - 2.0 ** -30, 1 - 1e-9, 1 - 1e-12, 1 - 2.0 ** -52, 1.0])
    for call in range(2):
        draws = np.concatenate([np.random.default_rng(300 + call).random(292), edge])
        d_draws = torch.from_numpy(draws).cuda()
        for rule, name in ((L.SAMPLE_BISECT, "bisect"), (L.SAMPLE_CDF, "cdf")):
            d_out = torch.full((len(draws),), -1, dtype=torch.int64, device="cuda")
            L.check(L.lib().qvmg_sample_noalloc(amps.data_ptr(), n, L.FP32,
                                                d_draws.data_ptr(), len(draws), rule,
                                                d_out.data_ptr(), stream.cuda_stream))
            stream.synchronize()
            got = d_out.cpu().numpy().astype(np.uint64)
            want = ref.sample(draws, rule=name)
            np.testing.assert_array_equal(got, want)
            assert got[-1] < (1 << n)
    ref.free()
    del amps
    torch.cuda.empty_cache()


def test_noalloc_rejects_states_beyond_its_scratch(gpu):
    with pytest.raises(L.QVMGError, match="outside 1..30"):
        L.check(L.lib().qvmg_sample_noalloc(1, 31, L.FP32, 1, 1, L.SAMPLE_BISECT, 1, None))
