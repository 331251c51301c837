"""The allocation-free line-opacity entry point, korg_line_absorption_noalloc (needs a GPU).

It exists for callers that cannot allocate device memory -- code running inside a memory pool
or arena it does not own, a process whose allocator is locked after start-up, or a caller in
the middle of stream capture.  It must give the same alpha as korg_line_absorption_dev, the
ordinary device-pointer entry point, call after call, even though every call reuses one
fixed device array for its scratch.  This file is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device_inputs(torch, inp, dev):
    from korg_gb300 import _lib
    keep = []

    def d(a, dt=torch.float64):
        t = torch.as_tensor(np.ascontiguousarray(a)).to(dt).to(dev)
        keep.append(t)
        return C.cast(t.data_ptr(), C.POINTER(C.c_double) if dt == torch.float64 else C.POINTER(C.c_int32))

    ll = inp.linelist
    lines = _lib.Lines(len(ll), d(ll.wl), d(ll.log_gf), d(ll.E_lower), d(ll.gamma_rad), d(ll.gamma_stark),
                       d(ll.vdW1), d(ll.vdW2), d(ll.mass), d(ll.is_mol, torch.int32), d(ll.species_idx, torch.int32))
    L = len(inp.T)
    lay = _lib.Layers(L, inp.n_div_U.shape[0], d(inp.T), d(inp.ne), d(inp.n_eff_vdW), d(inp.xi), d(inp.n_div_U))
    cn = _lib.Cntm(len(inp.cntm_knots), d(inp.cntm_knots), d(inp.cntm_vals))
    wls = torch.as_tensor(inp.wls.all_wls).to(dev)
    keep.append(wls)
    alpha0 = torch.as_tensor(np.stack([np.interp(inp.wls.all_wls, inp.cntm_knots, v) for v in inp.cntm_vals],
                                      axis=1)).to(dev)
    return lines, lay, cn, wls, alpha0, keep


def test_noalloc_matches_device_entry_point(gpu_lib):
    torch = pytest.importorskip("torch")
    from korg_gb300 import synthetic
    inp = synthetic.prepare(synthetic.config0())
    dev = torch.device("cuda:0")
    lines, lay, cn, wls, alpha0, keep = _device_inputs(torch, inp, dev)
    ctx = gpu_lib.Context(0)
    lib = ctx.lib
    stream = torch.cuda.current_stream(dev).cuda_stream
    for precision in (gpu_lib.KORG_FP64, gpu_lib.KORG_MIXED):
        ref = alpha0.clone()
        rc = lib.korg_line_absorption_dev(ctx.h, ref.data_ptr(), wls.data_ptr(), len(wls), C.byref(lines),
                                          C.byref(lay), C.byref(cn), inp.cutoff_threshold, precision, stream)
        assert rc == 0, lib.korg_last_error(ctx.h)
        torch.cuda.synchronize()
        ref = ref.cpu().numpy()
        assert np.any(ref != alpha0.cpu().numpy())  # lines were added
        for call in range(2):  # the second call reuses the array the first one left behind
            got = alpha0.clone()
            rc = lib.korg_line_absorption_noalloc(got.data_ptr(), wls.data_ptr(), len(wls), C.byref(lines),
                                                  C.byref(lay), C.byref(cn), inp.cutoff_threshold, precision,
                                                  stream)
            assert rc == 0, f"precision {precision}, call {call}: status {rc}"
            torch.cuda.synchronize()
            np.testing.assert_allclose(got.cpu().numpy(), ref, rtol=1e-9, atol=0)
    ctx.close()


def test_noalloc_rejects_problems_larger_than_its_array(gpu_lib):
    torch = pytest.importorskip("torch")
    from korg_gb300 import synthetic
    w = synthetic.config0(n_lines=100_000)  # 100k lines x 56 layers x 48 B of FP64 constants > 64 MiB
    inp = synthetic.prepare(w)
    dev = torch.device("cuda:0")
    lines, lay, cn, wls, alpha0, keep = _device_inputs(torch, inp, dev)
    got = alpha0.clone()
    rc = gpu_lib.lib().korg_line_absorption_noalloc(got.data_ptr(), wls.data_ptr(), len(wls), C.byref(lines),
                                                    C.byref(lay), C.byref(cn), inp.cutoff_threshold,
                                                    gpu_lib.KORG_FP64, torch.cuda.current_stream(dev).cuda_stream)
    assert rc == 5  # KORG_ETOOBIG
    torch.cuda.synchronize()
    assert torch.equal(got, alpha0)  # nothing was launched
