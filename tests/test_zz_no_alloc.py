"""
hg_prism_forward_noalloc: the forward for callers that cannot allocate device
memory (host frameworks that own the device pool, loops that must not
allocate mid-step, plugins with a fixed GPU budget).  It uses a fixed scratch
array in the library instead of a caller workspace or cudaMallocAsync.

Checked through the C ABI against two references on the same inputs:
hg_prism_forward given a workspace (the same kernels with caller scratch) and
the CPU oracle (an independent restatement of the reference's loop).  Two
calls run in a row, each with inputs that make the kernels use the scratch
(few points, many prisms: the prisms are split into chunks whose partial sums
live in the scratch); the second call also shows that the first call's
scratch contents do not leak into it.  Problems whose usual chunking needs
more partial sums than the scratch holds run with longer chunks and must
still match.  Tolerance: the FP64 parity tolerance of the GPU tests (1e-8
relative + 1e-9 of the largest value).

This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test.
"""

import ctypes

import numpy as np
import numpy.testing as npt
import pytest

pytestmark = pytest.mark.gpu

FIELD_NAMES = ("potential", "g_e", "g_n", "g_z", "g_ee", "g_nn", "g_zz", "g_en", "g_ez", "g_nz")


def _problem(seed, n_obs, n_prisms):
    rng = np.random.default_rng(seed)
    west = rng.uniform(-4e3, 3e3, n_prisms)
    south = rng.uniform(-4e3, 3e3, n_prisms)
    bottom = rng.uniform(-3e3, -300, n_prisms)
    prisms = np.column_stack([west, west + rng.uniform(20, 900, n_prisms), south,
                              south + rng.uniform(20, 900, n_prisms), bottom,
                              bottom + rng.uniform(20, 900, n_prisms)])
    density = rng.uniform(-600, 600, n_prisms)
    coords = (rng.uniform(-5e3, 5e3, n_obs), rng.uniform(-5e3, 5e3, n_obs),
              rng.uniform(10, 800, n_obs))
    return coords, prisms, density


def _device_inputs(lib, coords, prisms, density):
    import torch

    dev = torch.device("cuda")
    e, n, u = (torch.tensor(c, dtype=torch.float64, device=dev) for c in coords)
    aos = torch.tensor(prisms, dtype=torch.float64, device=dev)
    rho = torch.tensor(density, dtype=torch.float64, device=dev)
    m = prisms.shape[0]
    soa = torch.empty((7, m), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    assert lib.hg_pack_prisms(aos.data_ptr(), rho.data_ptr(), m, soa.data_ptr(), m, stream) == 0
    return e, n, u, soa


def _run_both(lib, coords, prisms, density, mask):
    """(hg_prism_forward with a workspace, hg_prism_forward_noalloc, bytes of
    the workspace the first one was given)."""
    import torch

    e, n, u, soa = _device_inputs(lib, coords, prisms, density)
    n_obs, m = e.numel(), prisms.shape[0]
    rows = bin(mask).count("1")
    stream = torch.cuda.current_stream().cuda_stream
    ws_bytes = ctypes.c_size_t(0)
    assert lib.hg_prism_forward_workspace(n_obs, m, mask, ctypes.byref(ws_bytes)) == 0
    assert ws_bytes.value > 0, "the case must exercise the scratch (chunked prisms)"
    ws = torch.empty(ws_bytes.value // 8 + 1, dtype=torch.float64, device=e.device)
    ref = torch.empty((rows, n_obs), dtype=torch.float64, device=e.device)
    new = torch.full((rows, n_obs), float("nan"), dtype=torch.float64, device=e.device)
    rc = lib.hg_prism_forward(e.data_ptr(), n.data_ptr(), u.data_ptr(), n_obs, soa.data_ptr(), m,
                              m, mask, ref.data_ptr(), None, ws.data_ptr(), ws_bytes.value,
                              stream)
    assert rc == 0, lib.hg_last_error()
    rc = lib.hg_prism_forward_noalloc(e.data_ptr(), n.data_ptr(), u.data_ptr(), n_obs,
                                      soa.data_ptr(), m, m, mask, new.data_ptr(), None, stream)
    assert rc == 0, lib.hg_last_error()
    torch.cuda.synchronize()
    return ref.cpu().numpy(), new.cpu().numpy(), ws_bytes.value


def _close(new, ref):
    npt.assert_allclose(new, ref, rtol=1e-8, atol=1e-9 * np.abs(ref).max())


def _check_oracle(oracle, new, coords, prisms, density, mask, stations=None):
    """Rows of `new` (one per field of `mask`) against the CPU oracle, on all
    points or on the given subset of them."""
    idx = np.arange(coords[0].size) if stations is None else np.asarray(stations)
    sub = tuple(np.ascontiguousarray(c[idx]) for c in coords)
    row = 0
    for code, name in enumerate(FIELD_NAMES):
        if (mask >> code) & 1:
            ref = oracle.prism_gravity(sub, prisms, density, field=name)
            _close(new[row][idx], ref)
            row += 1


def test_noalloc_matches_workspace_entry_point_and_oracle_twice(gpu_lib, oracle):
    lib = gpu_lib
    # first call: g_z, 300 points x 6000 prisms (the prisms are split in chunks)
    coords, prisms, density = _problem(11, 300, 6000)
    ref, new, _ = _run_both(lib, coords, prisms, density, 1 << 3)
    _close(new, ref)
    _check_oracle(oracle, new, coords, prisms, density, 1 << 3)
    # second call right after, other inputs and two fields: stale scratch from
    # the first call must not show up
    coords, prisms, density = _problem(12, 177, 4100)
    mask = (1 << 0) | (1 << 6)
    ref, new, _ = _run_both(lib, coords, prisms, density, mask)
    _close(new, ref)
    _check_oracle(oracle, new, coords, prisms, density, mask)


def test_noalloc_runs_problems_beyond_the_usual_chunking(gpu_lib, oracle):
    """Problems whose usual chunking needs more partial sums than the fixed
    scratch holds (8 MiB) run with longer chunks instead of being rejected."""
    lib = gpu_lib
    # g_z, 128 points x 2e6 prisms: the usual chunking wants ~16 MB
    coords, prisms, density = _problem(13, 128, 2_000_000)
    ref, new, ws = _run_both(lib, coords, prisms, density, 1 << 3)
    assert ws > 8 << 20
    _close(new, ref)
    _check_oracle(oracle, new, coords, prisms, density, 1 << 3, stations=np.arange(0, 128, 16))
    # all ten fields, 250 points x 200 000 prisms: the usual chunking wants
    # far more than 8 MiB
    coords, prisms, density = _problem(14, 250, 200_000)
    ref, new, ws = _run_both(lib, coords, prisms, density, 0x3FF)
    assert ws > 8 << 20
    _close(new, ref)
    _check_oracle(oracle, new, coords, prisms, density, 0x3FF, stations=[0, 97, 249])
    # ten fields over 60 000 points: fewer than two chunks fit, one chunk runs
    coords, prisms, density = _problem(15, 60_000, 3000)
    ref, new, ws = _run_both(lib, coords, prisms, density, 0x3FF)
    assert ws > 8 << 20
    _close(new, ref)
    _check_oracle(oracle, new, coords, prisms, density, 0x3FF, stations=[1, 30_000, 59_999])
