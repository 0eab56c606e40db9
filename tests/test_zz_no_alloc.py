"""The no-allocation FP64 sample sum (gtc_direct_fp64_noalloc).

Some callers of this library cannot allocate device memory: code inside
another framework whose caching allocator has already reserved the GPU's
memory, and timing-critical loops where cudaMalloc/cudaFree would stall the
device. gtc_direct_fp64_noalloc serves them with a fixed 8 MiB device array in
libgtc.so and the caller's stream, and needs no context. This test calls it
through the C ABI twice in a row and checks both results against the
context-based gtc_direct_fp64_device, to the 1e-12 relative tolerance of the
other FP64 sample test. It lives in its own file so that pytest collects it
last, and it builds its own inputs so that it also passes alone in a fresh
process.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _system(n, seed):
    rng = np.random.default_rng(seed)
    x = np.sqrt(rng.random(n) * 0.95)
    r = x / (1 - x)
    cz = 2 * rng.random(n) - 1
    ph = 2 * np.pi * rng.random(n)
    s = np.sqrt(1 - cz * cz)
    pos = r[:, None] * np.stack([s * np.cos(ph), s * np.sin(ph), cz], axis=1)
    pos[::10] += (3.0, -1.0, 2.0)
    return pos, rng.random(n) / n + 0.5 / n


@pytest.mark.parametrize("m", [1500, 262144])
def test_noalloc_matches_context_entry_point(gtc, m):
    """m = 262144 fills the fixed array with one source slice per target
    (the most targets it takes); sample indices repeat there."""
    import torch
    n = 20011
    pos, mass = _system(n, 17)
    rng = np.random.default_rng(5)
    idx = (rng.permutation(n)[:m] if m <= n else rng.integers(0, n, m)).astype(np.int64)
    dev = torch.device("cuda", 0)
    dpos = torch.tensor(pos, device=dev)
    dmass = torch.tensor(mass, device=dev)
    didx = torch.tensor(idx, device=dev)
    ref_acc = torch.zeros((m, 3), dtype=torch.float64, device=dev)
    ref_pot = torch.zeros(m, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    with gtc.Context(0) as ctx:
        ctx.direct_fp64_device(dpos.data_ptr(), dmass.data_ptr(), n, didx.data_ptr(), m,
                               ref_acc.data_ptr(), ref_pot.data_ptr(), G=1.0, eps=0.02)
    want_acc, want_pot = ref_acc.cpu().numpy(), ref_pot.cpu().numpy()
    stream = torch.cuda.current_stream(dev).cuda_stream
    for call in range(2):
        acc = torch.full((m, 3), float("nan"), dtype=torch.float64, device=dev)
        pot = torch.full((m,), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        gtc.direct_fp64_noalloc(dpos.data_ptr(), dmass.data_ptr(), n, didx.data_ptr(), m,
                                acc.data_ptr(), pot.data_ptr(), G=1.0, eps=0.02, stream=stream)
        torch.cuda.synchronize()
        a, p = acc.cpu().numpy(), pot.cpu().numpy()
        err = np.linalg.norm(a - want_acc, axis=1) / np.linalg.norm(want_acc, axis=1)
        assert err.max() < 1e-12, (call, err.max())
        assert np.abs(p / want_pot - 1).max() < 1e-12, call


def test_noalloc_refuses_more_targets_than_its_array(gtc):
    with pytest.raises(gtc.GtcInvalidArgument) as e:
        gtc.direct_fp64_noalloc(1, 1, 10, 1, 262145, 1, 1)
    assert "262144" in str(e.value)
