"""tapgpu_sssp_labels_noalloc: the entry point for callers that cannot let the
library allocate device memory (their own pool owns the HBM, or they cannot
afford the device synchronisation a cudaMalloc/cudaFree may cause).  It is
called through the C ABI on device buffers the test owns (torch tensors) and
must give the same labels as the allocating entry point tapgpu_sssp, bit for
bit (FP64 labels, the tolerance of the other label tests), on two calls in a
row: the shared fixed scratch array keeps the previous call's contents, so
the second call checks that nothing stale leaks into it.  Kept in a file that
pytest collects last."""

import numpy as np
import pytest

from traffic_assignment_gb300 import Solver, _capi, synth

pytestmark = pytest.mark.gpu


def _device_inputs(net, torch):
    va, ea = net.csr()
    dev = torch.device("cuda:0")
    row_ptr = torch.as_tensor(va.astype(np.int32), device=dev)
    head = torch.as_tensor(ea.astype(np.int32), device=dev)
    return row_ptr, head


def _call(lib, net, row_ptr, head, w, src, out, torch):
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.tapgpu_sssp_labels_noalloc(net.num_nodes + 1, net.num_links, net.first_thru_node,
                                        row_ptr.data_ptr(), head.data_ptr(), w.data_ptr(),
                                        src.data_ptr(), src.numel(), out.data_ptr(), stream)
    torch.cuda.synchronize()
    return rc


def test_noalloc_labels_match_allocating_entry_point(built_lib):
    torch = pytest.importorskip("torch")
    lib = built_lib
    net, _ = synth.make_grid3600()
    dev = torch.device("cuda:0")
    row_ptr, head = _device_inputs(net, torch)
    rng = np.random.default_rng(17)
    with Solver(net, None, precision="fp64") as s:
        for call in range(2):
            w_h = net.fft * rng.uniform(0.5, 2.0, net.num_links)
            src_h = np.sort(rng.choice(np.arange(1, net.num_nodes + 1), 40 + 23 * call,
                                       replace=False)).astype(np.int32)
            ref, _ = s.sssp(w_h, src_h, want_pred=False)
            w = torch.as_tensor(w_h, device=dev)
            src = torch.as_tensor(src_h, device=dev)
            out = torch.full((len(src_h), net.num_nodes + 1), -1.0, dtype=torch.float64,
                             device=dev)
            assert _call(lib, net, row_ptr, head, w, src, out, torch) == _capi.TAPGPU_OK
            got = out.cpu().numpy()
            got[np.isinf(got)] = np.finfo(np.float64).max
            np.testing.assert_array_equal(got, ref)


def test_noalloc_rejects_bad_input(built_lib):
    """Indices and weights in the caller's device memory are checked on the
    device before use: a source, a head or a weight out of range returns
    TAPGPU_ERR_ARG and leaves the output untouched; the next good call is
    unaffected by the failed one."""
    torch = pytest.importorskip("torch")
    lib = built_lib
    net, _ = synth.make_small24()
    dev = torch.device("cuda:0")
    row_ptr, head = _device_inputs(net, torch)
    w = torch.as_tensor(net.fft, device=dev)
    src = torch.as_tensor(np.array([1, 5], np.int32), device=dev)
    out = torch.full((2, net.num_nodes + 1), -7.0, dtype=torch.float64, device=dev)
    bad_src = torch.as_tensor(np.array([1, net.num_nodes + 5], np.int32), device=dev)
    assert _call(lib, net, row_ptr, head, w, bad_src, out, torch) == _capi.TAPGPU_ERR_ARG
    bad_head = head.clone()
    bad_head[3] = net.num_nodes + 3
    assert _call(lib, net, row_ptr, bad_head, w, src, out, torch) == _capi.TAPGPU_ERR_ARG
    bad_w = w.clone()
    bad_w[7] = -1.0
    assert _call(lib, net, row_ptr, head, bad_w, src, out, torch) == _capi.TAPGPU_ERR_ARG
    bad_rows = row_ptr.clone()
    bad_rows[4] = bad_rows[5] + 1
    assert _call(lib, net, bad_rows, head, w, src, out, torch) == _capi.TAPGPU_ERR_ARG
    assert bool((out == -7.0).all()), "a refused call wrote labels"
    assert _call(lib, net, row_ptr, head, w, src, out, torch) == _capi.TAPGPU_OK
    with Solver(net, None, precision="fp64") as s:
        ref, _ = s.sssp(net.fft, np.array([1, 5]), want_pred=False)
    got = out.cpu().numpy()
    got[np.isinf(got)] = np.finfo(np.float64).max
    np.testing.assert_array_equal(got, ref)
    # a graph too large for the fixed scratch array is refused before any launch
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.tapgpu_sssp_labels_noalloc(8_000_000, net.num_links, 1, row_ptr.data_ptr(),
                                        head.data_ptr(), w.data_ptr(), src.data_ptr(), 1,
                                        out.data_ptr(), stream)
    assert rc == _capi.TAPGPU_ERR_UNSUPPORTED
