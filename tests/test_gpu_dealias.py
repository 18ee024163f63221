"""GPU: padded (3/2-rule dealiased) Fourier transforms
(TensorProductSpace.get_dealiased, fourier/bases.py:409-435, 570-598)
against the reference's own results (golden fixture), both forms."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg():
    from shenfun_gb300 import build
    build.build()
    import shenfun_gb300
    return shenfun_gb300


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else a
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.parametrize("shape", [(8, 8, 17), (9, 7, 12)])
@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_dealiased_transforms(sg, golden, shape, form):
    d = golden("dealias")
    tag = "%dx%dx%d" % shape
    T = sg.TensorProductSpace(None, (sg.FunctionSpace(shape[0], "F", dtype="D"),
                                     sg.FunctionSpace(shape[1], "F", dtype="d"),
                                     sg.FunctionSpace(shape[2], "C", bc=(0, 0))), form=form)
    TD = T.get_dealiased((1.5, 1.5, 1))
    assert TD.shape(False) == d[f"{tag}_padded_in"].shape
    assert TD.shape(True) == d[f"{tag}_u_hat"].shape
    tol = 1e-12 if form == "plain" else 1e-10
    u_hat = sg.Function(TD, buffer=d[f"{tag}_u_hat"])
    assert rel(u_hat.backward(), d[f"{tag}_padded_backward"]) < tol
    b = sg.Array(TD, buffer=d[f"{tag}_padded_in"])
    assert rel(b.forward(), d[f"{tag}_padded_forward"]) < tol
    assert rel(sg.inner(sg.TestFunction(TD), b), d[f"{tag}_padded_scalar"]) < tol


def test_dealiased_product(sg):
    """The 3/2 rule removes aliasing from a quadratic product: the padded
    product of two band-limited fields, truncated, equals the exact product's
    coefficients within the retained modes (computed on a grid fine enough)."""
    N = 16
    T = sg.TensorProductSpace(None, (sg.FunctionSpace(N, "F", dtype="D"), sg.FunctionSpace(N, "F", dtype="d"),
                                     sg.FunctionSpace(17, "C", bc=(0, 0))))
    TD = T.get_dealiased((1.5, 1.5, 1))
    TF = T.get_dealiased((4, 4, 1))   # exact for the product of two N-mode fields
    rng = np.random.default_rng(0)
    a = sg.Array(T, buffer=rng.standard_normal(T.shape(False)))
    u_hat = a.forward()
    u_hat.v[:, :, -2:] = 0
    # zero the Nyquist modes so that the truncations agree exactly
    u_hat.v[N // 2] = 0
    u_hat.v[:, -1] = 0
    for S in (TD, TF):
        uh = sg.Function(S)
        uh.v.copy_(u_hat.v)
        up = uh.backward()
        up.v.mul_(up.v)
        out = up.forward()
        if S is TD:
            dealiased = out.v.clone()
        else:
            exact = out.v.clone()
    assert rel(dealiased, exact.cpu().numpy()) < 1e-12
