"""The allocation-free kokkosICP entry point (ss_kokkos_icp_noalloc) against
the allocating one (ss_kokkos_icp), through the C-ABI, on two calls in a row.

It exists for callers that cannot allocate device memory while they run
(a real-time tracking thread, or a process whose device memory belongs to its
own pool allocator); its scratch is a static device array, so every call must
give the same transform and RMSE as the allocating entry point (within the
tolerance of the parity tests: 1e-4 in the matrix, 1e-3 relative RMSE; the
two may reduce over a different number of CTAs), and a warm call must leave
the device's free memory unchanged. This file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

INTR = (525.0, 525.0, 319.5, 239.5)


def test_no_alloc_kokkos_icp_matches_allocating_entry_point():
    import torch
    import synth
    from superscanner_gb300._native import SS_ERR_DIMS, f64x16, lib
    sc = synth.Scene(1, 1234)
    P = sc.trajectory(20, 42)
    depth, _ = sc.render(P[[4, 6, 9]], 480, 640, INTR, noise=True, noise_seed=7, color=False)
    dev = [torch.from_numpy(np.ascontiguousarray(d.view(np.int16))).cuda() for d in depth]
    stream = torch.cuda.current_stream().cuda_stream

    def call(fn, a, b, ta, tb, kind):
        out = (C.c_double * 16)()
        rmse = C.c_float()
        st = fn(C.c_void_p(dev[a].data_ptr()), C.c_void_p(dev[b].data_ptr()), 480, 640, *INTR, f64x16(ta),
                f64x16(tb), kind, out, C.byref(rmse), C.c_void_p(stream))
        assert st == 0, st
        return np.array(out[:]).reshape(4, 4), rmse.value

    cases = [(0, 1, P[4], P[4], 1), (1, 2, P[6], P[6], 0)]  # two calls in a row, different inputs
    for q, (a, b, ta, tb, kind) in enumerate(cases):
        if q == 0:  # the allocation-free call first, before this case's allocating call
            T_new, r_new = call(lib.ss_kokkos_icp_noalloc, a, b, ta, tb, kind)
            T_ref, r_ref = call(lib.ss_kokkos_icp, a, b, ta, tb, kind)
        else:
            T_ref, r_ref = call(lib.ss_kokkos_icp, a, b, ta, tb, kind)
            T_new, r_new = call(lib.ss_kokkos_icp_noalloc, a, b, ta, tb, kind)
        assert np.abs(T_new - T_ref).max() < 1e-4
        assert r_new == pytest.approx(r_ref, rel=1e-3)
        assert np.abs(T_ref - np.eye(4)).max() > 1e-5  # the frames moved: a real alignment, not identity

    # the property the entry point exists for: a warm call leaves the device's free memory as it was
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    T_again, _ = call(lib.ss_kokkos_icp_noalloc, 0, 1, P[4], P[4], 1)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert np.abs(T_again - call(lib.ss_kokkos_icp, 0, 1, P[4], P[4], 1)[0]).max() < 1e-4

    # images above the 640 x 480 scratch are refused before any device work
    out = (C.c_double * 16)()
    rmse = C.c_float()
    st = lib.ss_kokkos_icp_noalloc(C.c_void_p(dev[0].data_ptr()), C.c_void_p(dev[1].data_ptr()), 481, 640, *INTR,
                                   f64x16(P[4]), f64x16(P[4]), 0, out, C.byref(rmse), C.c_void_p(stream))
    assert st == SS_ERR_DIMS
