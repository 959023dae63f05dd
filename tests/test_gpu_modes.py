"""GPU: mode decomposition kernels (lp_modes_project / lp_modes_combine) and
the Beam2D methods built on them, against the reference's outputs."""
import numpy as np
import pytest
import torch

from oracle import lp_oracle as O

pytestmark = pytest.mark.gpu
um, nm = O.um, O.nm


@pytest.fixture(scope="module")
def lp():
    import lightprop2d_gb300 as lp
    return lp


def beam(lp, golden):
    b = lp.Beam2D(96 * um, 64, 1064 * nm, init_field=golden["modes_field"])
    return b


def rel(a, b):
    a, b = np.asarray(a, np.complex128), np.asarray(b, np.complex128)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_deconstruct_construct_match_reference(lp, golden):
    m = golden["modes_basis"]
    b = beam(lp, golden)
    assert rel(b.deconstruct_by_modes(m), golden["modes_scalar"]) < 1e-6
    assert rel(b.modes_coeffs, golden["modes_scalar"]) < 1e-6
    assert rel(b.deconstruct_by_modes(m, "lstsq"), golden["modes_lstsq"]) < 1e-5
    mt = np.vstack(m).T
    assert rel(b.fast_deconstruct_by_modes(mt.T, mt.T.dot(mt)), golden["modes_fast"]) < 1e-5
    b.construct_by_modes(m, golden["modes_scalar"] * np.exp(0.5j))
    assert rel(b.field.cpu().numpy(), golden["modes_constructed"]) < 1e-6
    assert rel(b.spectrum.cpu().numpy(), golden["modes_constructed_spectrum"]) < 1e-5


@pytest.mark.parametrize("n,nb,M", [(512, 512, 40), (1024, 512, 64), (256, 64, 1000), (300, 98, 13)])
def test_project_combine_vs_oracle(lp, n, nb, M):
    from lightprop2d_gb300 import modes as MD
    rng = np.random.default_rng(n + M)
    modes = (rng.normal(size=(M, nb * nb)) + 1j * rng.normal(size=(M, nb * nb))) / nb
    f = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    basis = MD.ModeBasis(modes.astype(np.complex64))
    ft = torch.as_tensor(f.astype(np.complex64), device="cuda")
    c = MD.project(basis, ft).cpu().numpy()
    ref = O.modes_scalar(f.astype(np.complex64).astype(np.complex128),
                         modes.astype(np.complex64).astype(np.complex128))
    assert rel(c, ref) < 1e-6
    coef = rng.normal(size=M) + 1j * rng.normal(size=M)
    g = MD.combine(basis, coef, n, ft.device).cpu().numpy()
    gref = O.modes_combine(modes.astype(np.complex64).astype(np.complex128), coef, n)
    assert rel(g, gref) < 1e-6
    d = (n - nb) // 2
    if d:
        assert not np.any(g[:d]) and not np.any(g[:, :d])


def test_modes_errors(lp):
    from lightprop2d_gb300 import modes as MD
    basis = MD.ModeBasis(np.ones((3, 36)))
    with pytest.raises(ValueError):
        MD.project(basis, torch.ones((5, 5), dtype=torch.complex64, device="cuda"))
    with pytest.raises(ValueError):
        MD.combine(basis, [1, 2], 16, torch.device("cuda"))
    with pytest.raises(ValueError):
        MD.ModeBasis(np.ones((2, 35)))
    b = lp.Beam2D(96 * um, 64, 1064 * nm, init_field=np.ones((64, 64)))
    with pytest.raises(ValueError):
        b.deconstruct_by_modes(np.ones((2, 16)), mode="svd")
