"""The native drag adjoint against the pure-PyTorch FP64 reference and against
central finite differences (the adjoint's loss and gradients are defined in
include/lbm_gb300.h, lbm_adj_*).

Tolerances:
* FP64 run vs the PyTorch FP64 reference: loss 1e-11 and gradients 1e-8
  relative (two float64 evaluations of the same arithmetic in different orders);
* FP64 adjoint vs central differences of the FP64 forward run, step 1e-3 of
  each parameter: 1e-4 relative (the differences' own truncation error is
  ~1e-6 here);
* FP32 adjoint vs the FP64 adjoint: 1e-5 relative on the slice (measured
  5.5e-7), the accumulated float32 round-off of the forward and reverse
  sweeps over deviations f - w;
* at full size (256 x 128 x 32, 2000 steps): the FP32 and the FP64 adjoint
  both within 1e-4 of FP64 central differences (measured 4.1e-6, the
  differences' own truncation error), and within 2e-5 of each other
  (measured 1.5e-6).
"""

import numpy as np
import pytest
import torch

from oracle import diff_torch as D

# the 64 x 32 x 8 slice: cylinder r = 4 (width 1.5) at the reference placement
SLICE = dict(nx=64, ny=32, nz=8, steps=100, loss_start=51, r=4.0, width=1.5, u0=0.05, cs=0.1,
             reynolds=100.0)


def slice_model(steps=SLICE["steps"], loss_start=SLICE["loss_start"]):
    nx, ny, nz = SLICE["nx"], SLICE["ny"], SLICE["nz"]
    return D.Model(nx, ny, nz, steps=steps, loss_start=loss_start, ox=0.22 * nx, oy=0.5 * ny + 1.7,
                   width=SLICE["width"], diameter=2 * SLICE["r"], sponge_start=0.75 * nx)


def slice_params():
    d = 2 * SLICE["r"]
    return np.array([SLICE["u0"], 3 * SLICE["u0"] * d / SLICE["reynolds"] + 0.5, SLICE["cs"], SLICE["r"]])


def rel_err(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)) / np.maximum(np.abs(np.asarray(b)), 1e-300)


def test_torch_reference_matches_central_differences():
    """The reference gradient itself: autograd against central differences on a tiny lattice."""
    m = D.Model(16, 8, 4, steps=12, loss_start=7, ox=5.3, oy=3.6, width=1.5, diameter=5.0,
                sponge_start=12.0)
    p = [0.05, 0.53, 0.1, 2.5]
    _, g = D.gradient(m, p)
    fd = D.central_differences(m, p, 1e-4)
    assert rel_err(g, fd).max() < 1e-6


def make_run(precision, checkpoint=10, steps=SLICE["steps"], loss_start=SLICE["loss_start"]):
    from adjoint import DragAdjoint
    return DragAdjoint(SLICE["nx"], SLICE["ny"], SLICE["nz"], steps=steps, loss_start=loss_start,
                       checkpoint=checkpoint, precision=precision, u0=SLICE["u0"],
                       reynolds=SLICE["reynolds"], cs=SLICE["cs"], r=SLICE["r"], width=SLICE["width"])


@pytest.fixture(scope="module")
def reference():
    m = slice_model()
    return D.gradient(m, slice_params())


@pytest.mark.gpu
def test_fp64_adjoint_matches_torch_reference(reference):
    run = make_run("f64")
    assert np.allclose(run.params, slice_params(), rtol=0, atol=0)
    loss = run.forward()
    grad = run.backward()
    ref_loss, ref_grad = reference
    assert rel_err(loss, ref_loss) < 1e-11, (loss, ref_loss)
    assert rel_err(grad, ref_grad).max() < 1e-8, (grad, ref_grad)
    # the start state is lbm_init's equilibrium (lbm.py:383-394)
    m = slice_model()
    p = torch.tensor(slice_params())
    phi = 0.5 * (1 + torch.tanh((p[3] - m.d) / m.width))
    f0 = D.start_state(m, p[0], phi).numpy()
    assert np.abs(run.state(0) - f0).max() < 1e-15


@pytest.mark.gpu
def test_fp64_adjoint_matches_central_differences():
    run = make_run("f64")
    p0 = slice_params()
    run.forward()
    grad = run.backward()
    fd = np.zeros(4)
    for k in range(4):
        h = 1e-3 * abs(p0[k])
        lo, hi = p0.copy(), p0.copy()
        lo[k] -= h
        hi[k] += h
        run.set_params(hi)
        lh = run.forward()
        run.set_params(lo)
        ll = run.forward()
        fd[k] = (lh - ll) / (2 * h)
    assert rel_err(grad, fd).max() < 1e-4, (grad, fd)


@pytest.mark.gpu
def test_fp32_adjoint_against_fp64():
    r64, r32 = make_run("f64"), make_run("f32")
    l64, l32 = r64.forward(), r32.forward()
    g64, g32 = r64.backward(), r32.backward()
    assert rel_err(l32, l64) < 1e-6
    assert rel_err(g32, g64).max() < 1e-5, (g32, g64)


@pytest.mark.gpu
def test_checkpoint_interval_does_not_change_the_gradient():
    """Recomputation is exact: any checkpoint interval gives the same bits."""
    out = []
    for k in (1, 7, 100):
        run = make_run("f64", checkpoint=k)
        out.append((run.forward(), run.backward()))
    for loss, grad in out[1:]:
        assert loss == out[0][0]
        assert np.array_equal(grad, out[0][1])


@pytest.mark.gpu
def test_autograd_function():
    from adjoint import DragLoss
    run = make_run("f64")
    params = torch.tensor(slice_params(), dtype=torch.float64, requires_grad=True)
    loss = DragLoss.apply(params, run)
    (2.0 * loss).backward()
    run2 = make_run("f64")
    run2.forward()
    assert np.array_equal(params.grad.numpy(), 2.0 * run2.backward())


@pytest.mark.gpu
def test_autograd_two_applies_then_one_backward():
    """Two losses on one run before either backward: each gradient is its own."""
    from adjoint import DragLoss
    run = make_run("f64")
    p1 = torch.tensor(slice_params(), dtype=torch.float64, requires_grad=True)
    p2 = torch.tensor(slice_params() * np.array([1.02, 1.0, 1.1, 0.97]), dtype=torch.float64,
                      requires_grad=True)
    l1 = DragLoss.apply(p1, run)
    l2 = DragLoss.apply(p2, run)
    l1.backward()
    l2.backward()
    ref = make_run("f64")
    ref.forward()
    g1 = ref.backward()
    ref.set_params(p2.detach().numpy())
    ref.forward()
    g2 = ref.backward()
    assert np.array_equal(p1.grad.numpy(), g1)
    assert np.array_equal(p2.grad.numpy(), g2)
    assert not np.allclose(g1, g2)


@pytest.mark.gpu
def test_backward_needs_current_forward():
    import lbm_native as N
    run = make_run("f32")
    with pytest.raises(N.LbmError):
        run.backward()
    run.forward()
    run.set_params(slice_params() * 1.01)
    with pytest.raises(N.LbmError):
        run.backward()


@pytest.mark.gpu
@pytest.mark.slow
def test_full_size_adjoint_matches_central_differences():
    """256 x 128 x 32 LES cylinder at Re 100, 2000 steps, loss over steps
    1001..2000, checkpoints every 100 steps; r = 8, width 1.5, U = 0.05, Cs = 0.1.
    The FP64 and the FP32 adjoint against FP64 central differences
    (h = 1e-3 relative): 1e-4, the gradient tolerance the adjoint is held to."""
    from adjoint import DragAdjoint
    kw = dict(steps=2000, loss_start=1001, checkpoint=100, u0=0.05, reynolds=100.0, cs=0.1, r=8.0,
              width=1.5)
    r64 = DragAdjoint(256, 128, 32, precision="f64", **kw)
    p0 = r64.params.copy()
    r64.forward()
    g64 = r64.backward()
    fd = np.zeros(4)
    for k in range(4):
        h = 1e-3 * abs(p0[k])
        lo, hi = p0.copy(), p0.copy()
        lo[k] -= h
        hi[k] += h
        r64.set_params(hi)
        lh = r64.forward()
        r64.set_params(lo)
        ll = r64.forward()
        fd[k] = (lh - ll) / (2 * h)
    assert rel_err(g64, fd).max() < 1e-4, (g64, fd)
    del r64
    r32 = DragAdjoint(256, 128, 32, precision="f32", **kw)
    r32.forward()
    g32 = r32.backward()
    assert rel_err(g32, fd).max() < 1e-4, (g32, fd)
    assert rel_err(g32, g64).max() < 2e-5, (g32, g64)
