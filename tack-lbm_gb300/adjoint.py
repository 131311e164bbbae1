"""Gradients of time-averaged drag through the LES step (no reference counterpart).

``DragAdjoint`` runs the differentiable form of the step kept by the native
library (``lbm_adj_*`` in include/lbm_gb300.h): the cylinder along z is the
smoothed solid fraction ``phi = (1 + tanh((r - d)/width))/2``, used wherever
tack-lbm's step uses its 0/1 solid test (bounce-back, momentum exchange,
``u = fluid j / rho`` and the sponge, lbm.py:410-456), with LES-BGK collision
(lbm.py:72-93, 126-139), periodic boundaries and the lbm_init start state
(lbm.py:383-394). The loss is the drag coefficient averaged over the steps
``loss_start..steps``:

    L = sum_t F_x(t) / (N_l * 0.5 * U**2 * diameter * nz)

and its gradient with respect to ``(U, tau0, Cs, r)`` comes from the
hand-written adjoint kernel run backwards over the steps, each interval of
``checkpoint`` steps recomputed from the state the forward run kept.

``DragLoss`` is the ``torch.autograd.Function`` over it::

    run = DragAdjoint(256, 128, 32, steps=2000, loss_start=1001, checkpoint=100)
    params = torch.tensor([0.05, run.tau0, 0.1, 8.0], dtype=torch.float64, requires_grad=True)
    loss = DragLoss.apply(params, run)
    loss.backward()          # params.grad = dL/d(U, tau0, Cs, r)

PyTorch is the autograd plumbing only: the forward and backward passes are the
library's sm_103a kernels, and there is no fallback.
"""

import ctypes

import numpy as np
import torch

import lbm_native as N

PARAMS = ("u0", "tau0", "cs", "r")


class DragAdjoint:
    """One differentiable run: lattice, schedule and the current parameters.

    Defaults follow the reference Solver's placement (obstacle at
    (0.22 nx, 0.5 ny + 1.7), sponge from 0.75 nx with strength 1,
    lbm.py:561, lbm.py:630-637) and ``tau0 = 3 U D / Re + 1/2``.
    """

    def __init__(self, nx=256, ny=128, nz=32, *, steps=2000, loss_start=None, checkpoint=100,
                 precision="f32", u0=0.05, reynolds=100.0, tau0=None, cs=0.1, r=8.0, width=1.5,
                 center=None, diameter=None, sponge_start=None, sponge_strength=1.0, seed_amp=0.05,
                 device=0):
        c = N.AdjConfig()
        c.nx, c.ny, c.nz = nx, ny, nz
        c.precision = {"f32": N.F32, "f64": N.F64}[precision]
        c.steps = steps
        c.loss_start = steps // 2 + 1 if loss_start is None else loss_start
        c.checkpoint = checkpoint
        c.device = device
        self.diameter = 2.0 * r if diameter is None else diameter
        c.u0, c.cs, c.r = u0, cs, r
        c.tau0 = 3.0 * u0 * self.diameter / reynolds + 0.5 if tau0 is None else tau0
        cx, cy = (0.22 * nx, 0.5 * ny + 1.7) if center is None else center
        c.ox, c.oy, c.width = cx, cy, width
        c.diameter = self.diameter
        c.sponge_start = 0.75 * nx if sponge_start is None else sponge_start
        c.sponge_strength = sponge_strength
        c.seed_amp = seed_amp
        self.cfg = c
        self.lib = N.load()
        ptr = ctypes.c_void_p()
        N.check(self.lib.lbm_adj_create(ctypes.byref(c), ctypes.byref(ptr)))
        self.ptr = ptr
        self.params = np.array([c.u0, c.tau0, c.cs, c.r], np.float64)
        self.loss = None

    def __del__(self):
        ptr, self.ptr = getattr(self, "ptr", None), None
        if ptr and N._lib is not None:
            N._lib.lbm_adj_destroy(ptr)

    @property
    def tau0(self):
        return float(self.params[1])

    @property
    def n(self):
        return self.cfg.nx * self.cfg.ny * self.cfg.nz

    def set_params(self, params):
        """params = (U, tau0, Cs, r)."""
        p = np.ascontiguousarray(np.asarray(params, np.float64).reshape(4))
        N.check(self.lib.lbm_adj_set_params(self.ptr, p.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        self.params = p.copy()
        self.loss = None  # no forward pass at these parameters yet

    def forward(self):
        """Run all steps from the start state; returns the loss."""
        out = ctypes.c_double()
        N.check(self.lib.lbm_adj_forward(self.ptr, ctypes.byref(out)))
        self.loss = out.value
        return out.value

    def backward(self):
        """dL/d(U, tau0, Cs, r) of the last forward run, as a float64 array."""
        g = (ctypes.c_double * 4)()
        N.check(self.lib.lbm_adj_backward(self.ptr, g))
        return np.array(g[:], np.float64)

    def state(self, step):
        """Populations after ``step`` steps (a checkpointed step), shape (19, nz, ny, nx)."""
        dt = np.float64 if self.cfg.precision == N.F64 else np.float32
        out = np.empty((19, self.cfg.nz, self.cfg.ny, self.cfg.nx), dt)
        N.check(self.lib.lbm_adj_state(self.ptr, step, out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def info(self):
        """{forward_ms, backward_ms, force_sum, device_bytes} of the last runs."""
        v = (ctypes.c_double * 4)()
        N.check(self.lib.lbm_adj_info(self.ptr, v))
        return {"forward_ms": v[0], "backward_ms": v[1], "force_sum": v[2], "device_bytes": int(v[3])}


class DragLoss(torch.autograd.Function):
    """loss = DragLoss.apply(params, run): params = (U, tau0, Cs, r) as a 4-tensor.

    Each application keeps its own parameters. The run holds the checkpoints
    of its last forward pass only, so when ``run`` has been applied again at
    other parameters before this loss's ``backward`` (a line search, two
    losses in one graph), ``backward`` first reruns the forward pass at this
    application's parameters; the gradient is always that of this loss."""

    @staticmethod
    def forward(ctx, params, run):
        p = params.detach().to("cpu", torch.float64).numpy().copy()
        run.set_params(p)
        ctx.run = run
        ctx.params = p
        return params.new_tensor(run.forward())

    @staticmethod
    def backward(ctx, grad_out):
        run = ctx.run
        if run.loss is None or not np.array_equal(run.params, ctx.params):
            run.set_params(ctx.params)
            run.forward()
        g = torch.as_tensor(run.backward(), dtype=grad_out.dtype, device=grad_out.device)
        return grad_out * g, None


def drag_loss(params, run):
    """The time-averaged drag coefficient of ``run`` at ``params``, differentiable."""
    return DragLoss.apply(params, run)
