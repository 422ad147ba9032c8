"""The allocation-free pair sort (mpm_sort_pairs_noalloc) against the sort the substep
already runs inside a context (mpm_get_sort), through the C ABI, on two calls in a row.

Callers that cannot allocate device memory when they sort (a loop being recorded into a
CUDA graph, a real-time loop that cannot take cudaMalloc's synchronisation, a framework
that owns all device memory) hand their own device arrays to this entry point; its working
memory is a fixed static area shared by all calls on the GPU. This file is collected last
so a failure here comes after every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

from non_ficks_diffusion_gb300 import capi, workloads

pytestmark = pytest.mark.gpu


def _keys(X, counts):
    x = X.astype(np.float32)
    c = np.floor(x * np.array(counts, dtype=np.float32)).astype(np.int64) + 4
    b, l = c >> 2, c & 3
    nb = np.array(counts) // 4 + 2
    gb = b[:, 0] + nb[0] * (b[:, 1] + nb[1] * b[:, 2])
    return ((gb << 6) | l[:, 0] | (l[:, 1] << 2) | (l[:, 2] << 4)).astype(np.uint32)


def _context_sort(desc, parts):
    """The existing entry points: a context's first grid build sorts the particles."""
    ctx = capi.Context(precision="fp32", max_particles=len(parts["mass"]), max_scenes=1)
    sid = ctx.add_scene(desc)
    ctx.add_particles(sid, parts["X"], parts["V"], parts["mass"], parts["lambda0"], parts["mu0"])
    ctx.initialize()
    keys, order, _ = ctx.sort_state()
    ctx.close()
    return keys, order


def test_noalloc_sort_matches_context_sort_twice(built_lib):
    torch = pytest.importorskip("torch")
    L = capi.lib()
    scenes = [workloads.ball_scene(n=32, radius=0.12, seed=5),
              workloads.ball_scene(n=64, center=(0.4, 0.5, 0.55), radius=0.15, seed=9)]
    for desc, parts in scenes:                      # two calls in a row, different inputs
        ref_keys, ref_order = _context_sort(desc, parts)
        keys = _keys(parts["X"], list(desc.counts))
        n = len(keys)
        kin = torch.from_numpy(keys.view(np.int32)).cuda()
        kout = torch.empty_like(kin)
        vout = torch.empty(n, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        st = L.mpm_sort_pairs_noalloc(kin.data_ptr(), None, kout.data_ptr(), vout.data_ptr(), n, 6, 32, None)
        assert st == capi.OK
        torch.cuda.synchronize()
        got_keys = kout.cpu().numpy().view(np.uint32)
        got_order = vout.cpu().numpy()
        assert np.array_equal(got_keys, ref_keys)
        assert np.array_equal(got_order, ref_order)


def _expected(keys, vals, begin, end):
    """Stable order by the ceil((end-begin)/8) 8-bit digits from bit `begin` upward."""
    passes = (end - begin + 7) // 8
    digits = (keys.astype(np.uint64) >> np.uint64(begin)) & np.uint64((1 << (8 * passes)) - 1)
    perm = np.argsort(digits, kind="stable")
    return keys[perm], (vals[perm] if vals is not None else perm.astype(np.int32))


@pytest.mark.parametrize("n", [70001, 1 << 20])
def test_noalloc_sort_at_its_limit(built_lib, n):
    """Random 32-bit keys up to the documented maximum (n = 2^20: 256 tiles, a scan over
    65,536 digit counts in 16 segments), over 1, 3 and 4 digit passes (an odd count
    writes pass 0 to the caller's output), with and without caller values, called back to
    back on one stream: every call matches numpy's stable sort, so the shared static
    scratch carries nothing from one call into the next."""
    torch = pytest.importorskip("torch")
    L = capi.lib()
    rng = np.random.default_rng(n)
    cases = [(0, 8, False), (0, 24, True), (0, 32, False), (6, 32, True), (0, 32, True)]
    keys = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    keys[: n // 10] &= 0xFF00FF00          # many equal digits: stability matters
    vals = rng.integers(-(1 << 31), (1 << 31) - 1, n, dtype=np.int64).astype(np.int32)
    kin = torch.from_numpy(keys.view(np.int32)).cuda()
    vin = torch.from_numpy(vals).cuda()
    outs = []
    for begin, end, with_vals in cases:
        kout = torch.empty_like(kin)
        vout = torch.empty(n, dtype=torch.int32, device="cuda")
        st = L.mpm_sort_pairs_noalloc(kin.data_ptr(), vin.data_ptr() if with_vals else None, kout.data_ptr(),
                                      vout.data_ptr(), n, begin, end, None)
        assert st == capi.OK
        outs.append((kout, vout))
    torch.cuda.synchronize()
    for (begin, end, with_vals), (kout, vout) in zip(cases, outs):
        want_k, want_v = _expected(keys, vals if with_vals else None, begin, end)
        assert np.array_equal(kout.cpu().numpy().view(np.uint32), want_k), (begin, end, with_vals)
        assert np.array_equal(vout.cpu().numpy(), want_v), (begin, end, with_vals)


def test_noalloc_sort_limits(built_lib):
    L = capi.lib()
    assert L.mpm_sort_pairs_noalloc(None, None, None, None, 10, 0, 32, None) == capi.BAD_ARG
    torch = pytest.importorskip("torch")
    k = torch.zeros(8, dtype=torch.int32, device="cuda")
    v = torch.zeros(8, dtype=torch.int32, device="cuda")
    too_many = capi.lib().mpm_sort_pairs_noalloc(k.data_ptr(), None, k.data_ptr() + 32, v.data_ptr(),
                                                 (1 << 20) + 1, 0, 32, None)
    assert too_many == capi.BAD_ARG
    assert L.mpm_sort_pairs_noalloc(k.data_ptr(), None, k.data_ptr(), v.data_ptr(), 8, 0, 32, None) == capi.BAD_ARG
