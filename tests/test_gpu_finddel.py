"""findDelAuto on the GPU (sampHighOrder + setPhiDiv + cgne, coarse search through
cgne_batch) against the FP64 restatement (findDel/findDelAuto.m)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_find_del_auto_vs_restatement():
    import matmri_gb300 as mm
    from oracle.finddel_ref import find_del_auto
    from sho_cases import finddel_case
    c = finddel_case(N=16, C=3, M=768, true_delay=0.37, wobble=6.0)
    args = (c["data"], c["tdwell"], c["traj"], c["conc"], c["datatime"], c["grid"], c["b0"], c["maps"], 15)
    d, hist = mm.findDelAuto(0.0, *args)
    dr, hr = find_del_auto(0.0, *args)
    assert hist[0] == hr[0]                               # the same coarse-search pick
    assert abs(d - dr) < 0.01
    assert abs(d - c["true_delay"]) < 0.05
    n = min(len(hist), len(hr))
    assert abs(len(hist) - len(hr)) <= 1
    np.testing.assert_allclose(hist[:n], hr[:n], atol=0.01)


def test_find_del_auto_device_data_and_no_coarse_search():
    import torch
    import matmri_gb300 as mm
    from sho_cases import finddel_case
    c = finddel_case(N=16, C=3, M=768, true_delay=-0.6, wobble=6.0, seed=11)
    dd = torch.from_numpy(np.asfortranarray(c["data"]).astype(np.complex64)).cuda()
    args = (c["tdwell"], c["traj"], c["conc"], c["datatime"], c["grid"], c["b0"], c["maps"], 15)
    d_host, _ = mm.findDelAuto(0.0, c["data"].astype(np.complex64), *args, 3, 0)
    d_dev, h = mm.findDelAuto(0.0, dd, *args, 3, 0)
    assert h[0] == 0.0                                    # numCoarseSearch = 0 starts at delSk0
    assert abs(d_host - d_dev) < 1e-3
    assert abs(d_dev - c["true_delay"]) < 0.08
