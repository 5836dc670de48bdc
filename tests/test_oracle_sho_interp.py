"""Interpolated @sampHighOrder encoding (approach 1): the FP64 restatement pinned
against the reference's own test (@sampHighOrder/tests.m:66-147), and the
host-side plan of the product checked against the restatement."""
import numpy as np
import pytest

from oracle.sho_interp_ref import ShoInterpRef, filtnd_gauss, prep_for_interp, subsamp_time
from oracle.sho_ref import ShoRef
from sho_cases import interp_case, orient_grid

OPT = dict(svdThresh=0.01, subFact=5)          # tests.m:67-70


@pytest.fixture(scope="module")
def case():
    return interp_case(32, seed=1)


def _image(N0, seed=2):
    rng = np.random.default_rng(seed)
    img = np.zeros((N0, N0))
    yy, xx = np.mgrid[-1:1:N0 * 1j, -1:1:N0 * 1j]
    for _ in range(6):
        cx, cy, a, b = rng.uniform(-0.5, 0.5), rng.uniform(-0.5, 0.5), rng.uniform(0.1, 0.5), rng.uniform(0.1, 0.5)
        img += rng.uniform(0.2, 1.0) * (((xx - cx) / a) ** 2 + ((yy - cy) / b) ** 2 < 1)
    return img.astype(np.complex128)


@pytest.mark.parametrize("orient", [0, 1, 2, 3])
def test_interp_matches_direct_and_is_adjoint(case, orient):
    # tests.m:101-139: adjoint to 1e-8, and ||S_direct x - S_interp x|| / numel < 1e-4
    grid = orient_grid(case, orient)
    xvec = _image(case["N0"])
    rng = np.random.default_rng(3)
    yvec = rng.standard_normal(case["M"]) + 1j * rng.standard_normal(case["M"])
    Sx = ShoRef(case["b0"], case["t"], case["spha"], case["coco"], grid).mtimes(xvec).ravel()
    f = prep_for_interp(case["b0"], case["t"], case["spha"], case["coco"], grid, None, **OPT)
    S = ShoInterpRef([case["N0"]] * 2, f)
    Sxb = S.mtimes(xvec).ravel()
    Syb = S.H.mtimes(yvec).ravel(order="F")
    d1 = np.vdot(xvec.ravel(order="F"), Syb)
    d2 = np.vdot(Sxb, yvec)
    assert abs(d1 - d2) / min(abs(d1), abs(d2)) < 1e-8
    cost = np.linalg.norm(Sx - Sxb) / Sx.size
    assert cost < 1e-4
    # the truncation keeps the triplets up to and including the first below the threshold (tests.m:839)
    s = f["s"]
    assert s[-1] / s[0] < OPT["svdThresh"] <= s[-2] / s[0]


def test_interp_nd_sample_times(case):
    # tests.m:141-147: sampTimes [M/2, 2] gives the same encoding as the vector form
    grid = orient_grid(case, 0)
    M = case["M"]
    xvec = _image(case["N0"])
    f1 = prep_for_interp(case["b0"], case["t"], case["spha"], case["coco"], grid, None, **OPT)
    f2 = prep_for_interp(case["b0"], case["t"].reshape(-1, 2, order="F"),
                         case["spha"].reshape(16, -1, 2, order="F"), case["coco"].reshape(4, -1, 2, order="F"),
                         grid, None, **OPT)
    a = ShoInterpRef([case["N0"]] * 2, f1).mtimes(xvec).ravel()
    b = ShoInterpRef([case["N0"]] * 2, f2).mtimes(xvec).ravel()
    assert np.linalg.norm(a - b) / M < 1e-4


def test_gauss_window_and_subsampling():
    # filtNd(2*(h+1), 0.5, 1, 'gauss'): peak at index sz/2 (k-space centre), symmetric after dropping the first tap
    w = filtnd_gauss(8, 0.5)
    assert np.argmax(w) == 4 and w.max() == 1.0
    np.testing.assert_allclose(w[1:], w[1:][::-1], rtol=0, atol=1e-15)
    a = np.random.default_rng(0).standard_normal((3, 23))
    sp, cc, t, inds = subsamp_time(a, a[:1], np.arange(23.0), 5)
    assert list(inds) == [0, 5, 10, 15, 20, 22]                          # keeps the last sample
    np.testing.assert_array_equal(sp[:, 0], a[:, 0])                       # edge samples untouched
    np.testing.assert_array_equal(sp[:, -1], a[:, -1])
    const = np.ones((1, 23))
    sp, _, _, _ = subsamp_time(const, const, np.arange(23.0), 5)
    np.testing.assert_allclose(sp, 1.0, atol=1e-14)                        # unit-sum window


@pytest.mark.parametrize("randomized", [False, True])
@pytest.mark.parametrize("masked", [False, True])
def test_product_plan_matches_restatement(case, randomized, masked, monkeypatch):
    import matmri_gb300.sho_interp as si
    if randomized:
        monkeypatch.setattr(si, "EXACT_SVD_MAX", 8)
    grid = orient_grid(case, 1)
    mask = None
    if masked:
        mask = (case["x"] ** 2 + case["y"] ** 2) < (0.8 * np.abs(case["x"]).max()) ** 2
    a = si.prep_for_interp(case["b0"], case["t"], case["spha"], case["coco"], grid, mask, 0.01, 5)
    b = prep_for_interp(case["b0"], case["t"], case["spha"], case["coco"], grid, mask, 0.01, 5)
    assert a["s"].size == b["s"].size
    np.testing.assert_allclose(a["kloc"], b["kloc"], rtol=0, atol=1e-15)
    np.testing.assert_allclose(a["phsShft"], b["phsShft"], rtol=0, atol=1e-15)
    np.testing.assert_allclose(a["s"], b["s"], rtol=1e-12)
    Ea = a["svdSpace"] @ a["svdTime"].T
    Eb = b["svdSpace"] @ b["svdTime"].T
    assert np.abs(Ea - Eb).max() < 1e-10 * np.abs(Eb).max()
    if masked:
        assert np.all(a["svdSpace"][~mask.reshape(-1, order="F")] == 0)


def test_plan_rejects_unsupported_grids(case):
    import matmri_gb300.sho_interp as si
    grid = orient_grid(case, 0)
    tilted = dict(grid, z=grid["z"] + 0.01 * grid["x"])
    with pytest.raises(ValueError, match="non-axial"):
        si.prep_for_interp(case["b0"], case["t"], case["spha"], case["coco"], tilted)
    odd = {k: v[:-1, :-1] for k, v in grid.items()}
    with pytest.raises(ValueError, match="even"):
        si.prep_for_interp(case["b0"][:-1, :-1], case["t"], case["spha"], case["coco"], odd)
