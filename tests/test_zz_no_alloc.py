"""The allocation-free thermodynamic reduction (gb_thermo_reduce_noalloc) against the allocating
one (gb_thermo_reduce), through the C ABI.

gb_thermo_reduce_noalloc exists for callers that cannot allocate device memory -- a host whose
device memory belongs to its own pool, or one that must not stall the GPU with cudaFree -- and
therefore cannot pass the scratch buffer gb_thermo_reduce takes. It reduces through a fixed
array inside the library instead. This file is collected last so that a run stopping at the
first failure has already run every other test; it also passes on its own in a fresh process.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from hoomd_gb300 import abi  # noqa: E402


def _inputs(N, seed):
    rng = np.random.default_rng(seed)
    vel = np.zeros((N, 4), np.float32)
    vel[:, :3] = rng.normal(0, 1.3, (N, 3))
    vel[:, 3] = rng.uniform(0.5, 2.0, N)
    force = rng.normal(0, 5, (N, 4)).astype(np.float32)
    virial = rng.normal(0, 2, (6, N)).astype(np.float32)
    return [torch.from_numpy(a).cuda() for a in (vel, force, virial)]


def test_no_alloc_reduction_matches_allocating_reduction_twice():
    lib = abi.load()
    stream = torch.cuda.current_stream().cuda_stream
    for call, (N, seed) in enumerate([(300001, 1), (4096, 2)]):
        vel, force, virial = _inputs(N, seed)
        scratch = torch.zeros(lib.gb_thermo_scratch_bytes(N), dtype=torch.uint8, device="cuda")
        want = torch.zeros(3, dtype=torch.float64, device="cuda")
        got = torch.full((3,), np.nan, dtype=torch.float64, device="cuda")
        abi.check(lib.gb_thermo_reduce(vel.data_ptr(), force.data_ptr(), virial.data_ptr(), N,
                                       N, scratch.data_ptr(), want.data_ptr(), stream),
                  "gb_thermo_reduce")
        abi.check(lib.gb_thermo_reduce_noalloc(vel.data_ptr(), force.data_ptr(),
                                               virial.data_ptr(), N, N, got.data_ptr(), stream),
                  "gb_thermo_reduce_noalloc")
        torch.cuda.synchronize()
        w, g = want.cpu().numpy(), got.cpu().numpy()
        # same terms and the same fixed-order reduction: equal to FP64 round-off
        assert np.allclose(g, w, rtol=1e-12, atol=1e-9), (call, g, w)
        v = vel.cpu().numpy().astype(np.float64)
        ke = 0.5 * np.sum(v[:, 3] * (v[:, :3] ** 2).sum(1))
        assert np.isclose(g[0], ke, rtol=1e-12)


def test_no_alloc_rejects_too_many_particles():
    lib = abi.load()
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    dummy = torch.zeros(4, dtype=torch.float32, device="cuda")
    rc = lib.gb_thermo_reduce_noalloc(dummy.data_ptr(), None, None, 0, 4194305, out.data_ptr(),
                                      torch.cuda.current_stream().cuda_stream)
    assert rc == abi.GB_ERR_TOO_LARGE
    assert b"GB_NOALLOC_MAX_N" in lib.gb_last_error()
