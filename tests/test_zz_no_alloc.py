"""The allocation-free line-opacity entry point, korg_line_absorption_noalloc (needs a GPU).

It exists for callers that cannot allocate device memory -- code running inside a memory pool
or arena it does not own, a process whose allocator is locked after start-up, or a caller in
the middle of stream capture.  It must give the same alpha as korg_line_absorption_dev, the
ordinary device-pointer entry point, call after call, even though every call reuses one
fixed device array for its scratch.  Both run the same kernels with the same tile shape, so
the results must be bitwise equal: a value left behind in the shared array (a stale counter or
sortedness flag that changed the order of additions) would show up here.  This file is named so
that pytest collects it last.
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
            np.testing.assert_array_equal(got.cpu().numpy(), ref)
    ctx.close()


def _noalloc(lib, alpha, wls, lines, lay, cn, inp, precision, stream):
    return lib.korg_line_absorption_noalloc(alpha.data_ptr(), wls.data_ptr(), len(wls), C.byref(lines), C.byref(lay),
                                            C.byref(cn), inp.cutoff_threshold, precision, stream)


def test_noalloc_under_stream_capture(gpu_lib):
    """A caller in the middle of stream capture: after one ordinary call (the per-context set-up),
    a call captured into a CUDA graph on a side stream replays to the device entry point's alpha."""
    torch = pytest.importorskip("torch")
    from korg_gb300 import synthetic
    w = synthetic.config0(n_lines=600)
    w.wavelengths = (5000, 5040)
    inp = synthetic.prepare(w)
    dev = torch.device("cuda:0")
    lines, lay, cn, wls, alpha0, keep = _device_inputs(torch, inp, dev)
    ctx = gpu_lib.Context(0)
    lib = ctx.lib
    main = torch.cuda.current_stream(dev)
    for precision in (gpu_lib.KORG_MIXED, gpu_lib.KORG_FP64):
        ref = alpha0.clone()
        assert lib.korg_line_absorption_dev(ctx.h, ref.data_ptr(), wls.data_ptr(), len(wls), C.byref(lines),
                                            C.byref(lay), C.byref(cn), inp.cutoff_threshold, precision,
                                            main.cuda_stream) == 0
        got = alpha0.clone()
        assert _noalloc(lib, got, wls, lines, lay, cn, inp, precision, main.cuda_stream) == 0  # set-up call
        torch.cuda.synchronize()
        ref = ref.cpu().numpy()
        np.testing.assert_array_equal(got.cpu().numpy(), ref)
        graph = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream(dev)
        side.wait_stream(main)
        rcs = []
        with torch.cuda.graph(graph, stream=side):
            rcs.append(_noalloc(lib, got, wls, lines, lay, cn, inp, precision, side.cuda_stream))
        assert rcs == [0]
        for replay in range(2):
            got.copy_(alpha0)
            graph.replay()
            torch.cuda.synchronize()
            np.testing.assert_array_equal(got.cpu().numpy(), ref, err_msg=f"precision {precision}, replay {replay}")
        del graph
    ctx.close()


def test_noalloc_rejects_problems_larger_than_its_array(gpu_lib):
    torch = pytest.importorskip("torch")
    from korg_gb300 import synthetic
    # 100k lines x 56 layers: 48 B of FP64 constants (269 MB) or 32 B of mixed ones (179 MB) per
    # line and layer, both above the 64 MiB array
    w = synthetic.config0(n_lines=100_000)
    inp = synthetic.prepare(w)
    dev = torch.device("cuda:0")
    lines, lay, cn, wls, alpha0, keep = _device_inputs(torch, inp, dev)
    lib = gpu_lib.lib()
    stream = torch.cuda.current_stream(dev).cuda_stream
    for precision in (gpu_lib.KORG_FP64, gpu_lib.KORG_MIXED):
        got = alpha0.clone()
        assert _noalloc(lib, got, wls, lines, lay, cn, inp, precision, stream) == 5  # KORG_ETOOBIG
        torch.cuda.synchronize()
        assert torch.equal(got, alpha0)  # nothing was launched
    got = alpha0.clone()
    assert _noalloc(lib, got, wls, lines, lay, cn, inp, 2, stream) == 1  # KORG_EINVAL: not a precision
