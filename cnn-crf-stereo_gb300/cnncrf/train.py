"""The training step over the C ABI (cnncrf_train_*) and its autograd form.

Trainer drives the library's fused step: forward through both nets and the
correlation, the structured hinge on the CRF's loss-augmented labelling, the
hand-written adjoints, SGD with momentum on FP32 master weights.

StereoNetsFunction and HingeLossFunction are thin torch.autograd.Functions
over the same calls, so a torch training loop can own the parameters and the
optimizer:

    vol, pw = StereoNetsFunction.apply(trainer, left, right, *params)
    loss = HingeLossFunction.apply(trainer, vol, pw, gt)
    loss.backward()          # the library's adjoints fill params[i].grad

The reference ships no training code (its weights were trained elsewhere).
"""
import ctypes as C
import os

import numpy as np
import torch

from . import _lib as L
from ._lib import TrainDesc, call
from .api import _ptr, _stream_ptr, as_device_tensor


def _count(dmin, dstep, dmax):
    """The float loop of the stored list: d = dmin; d <= dmax; d += dstep."""
    n, d = 0, np.float32(dmin)
    while d <= np.float32(dmax):
        n += 1
        d = np.float32(d + np.float32(dstep))
    return n


class Trainer:
    def __init__(self, npairs, width, height, num_layers=7, topology=L.TOPO_ALL3X3, feat_channels=100,
                 pw_channels=64, disp_min=0.0, disp_step=1.0, disp_max=127.0, lam=1.0, L1=0.5, L2=1.5, delta=3,
                 crf_shape=L.RHO_LINEAR, crf_slack=0.5, crf_iters=8, mean_loss=True, precision=L.BF16,
                 checkpoint_every=3, tc_wgrad=True, tc_dgrad=True, stream=None):
        d = TrainDesc()
        call("cnncrf_train_default_desc", C.byref(d))
        d.num_layers, d.topology, d.feat_channels, d.pw_channels = num_layers, topology, feat_channels, pw_channels
        d.disp_min, d.disp_step, d.disp_max, d.lam = disp_min, disp_step, disp_max, lam
        d.L1, d.L2, d.delta, d.crf_shape, d.crf_slack, d.crf_iters = L1, L2, delta, crf_shape, crf_slack, crf_iters
        d.mean_loss = 1 if mean_loss else 0
        d.precision, d.checkpoint_every = precision, checkpoint_every
        d.tc_wgrad = 1 if tc_wgrad else 0
        d.tc_dgrad = 1 if tc_dgrad else 0
        self._h = C.c_void_p()
        call("cnncrf_train_create", C.byref(self._h), C.byref(d), npairs, width, height)
        self.stream = stream
        call("cnncrf_train_set_stream", self._h, _stream_ptr(stream))
        self.n, self.W, self.H = npairs, width, height
        self.D = _count(disp_min, disp_step, disp_max)
        self.mean_loss = bool(mean_loss)

    def __del__(self):
        if getattr(self, "_h", None) and L._lib is not None:
            L.lib().cnncrf_train_destroy(self._h)
            self._h = None

    # ---- parameters (npz slot order and shapes)
    def num_params(self):
        n = C.c_int()
        call("cnncrf_train_num_params", self._h, C.byref(n))
        return n.value

    def param_shape(self, i):
        s = (C.c_int64 * 4)()
        nd = C.c_int()
        call("cnncrf_train_param_shape", self._h, i, s, C.byref(nd))
        return tuple(s[k] for k in range(nd.value))

    def init_xavier(self, seed=0):
        call("cnncrf_train_init_xavier", self._h, seed)

    def save(self, path):
        """Checkpoint: weights as arr_i (a parameter file for inference too) and momentum as mom_i."""
        call("cnncrf_train_save", self._h, os.fsencode(path))

    def load(self, path):
        """Resume from save()'s file, or start from a plain parameter file (zero momentum)."""
        call("cnncrf_train_load", self._h, os.fsencode(path))

    def set_param(self, i, a):
        """Host array or CUDA tensor of the slot's shape."""
        if isinstance(a, torch.Tensor) and a.is_cuda:
            a = a.detach().contiguous().float()
            call("cnncrf_train_set_param", self._h, i, _ptr(a), a.numel())
            return
        a = np.ascontiguousarray(a, np.float32)
        call("cnncrf_train_set_param", self._h, i, a.ctypes.data_as(C.c_void_p), a.size)

    def get_param(self, i):
        out = np.empty(self.param_shape(i), np.float32)
        call("cnncrf_train_get_param", self._h, i, out.ctypes.data_as(C.c_void_p), out.size)
        return out

    def get_grad(self, i):
        out = np.empty(self.param_shape(i), np.float32)
        call("cnncrf_train_get_grad", self._h, i, out.ctypes.data_as(C.c_void_p), out.size)
        return out

    def grad_tensor(self, i):
        out = torch.empty(self.param_shape(i), device="cuda", dtype=torch.float32)
        call("cnncrf_train_get_grad", self._h, i, _ptr(out), out.numel())
        return out

    # ---- the step's parts
    def forward(self, left, right):
        """left, right: CUDA [n][H][W][4] RGBA; returns views of the unary
        volume [n][H][W][D] and the pairwise output |h| [n][2][H][W]."""
        left, right = left.contiguous(), right.contiguous()
        call("cnncrf_train_forward", self._h, _ptr(left), _ptr(right))
        return self.outputs()

    def outputs(self):
        v, p, d = C.c_void_p(), C.c_void_p(), C.c_int()
        call("cnncrf_train_outputs", self._h, C.byref(v), C.byref(p), C.byref(d))
        return (as_device_tensor(v.value, (self.n, self.H, self.W, d.value)),
                as_device_tensor(p.value, (self.n, 2, self.H, self.W)))

    def hinge(self, gt):
        """gt: CUDA int32 [n][H][W] labels; returns the per-pair losses and y^."""
        gt = gt.contiguous()
        loss = (C.c_double * self.n)()
        yh = torch.empty((self.n, self.H, self.W), device="cuda", dtype=torch.int32)
        call("cnncrf_train_hinge", self._h, _ptr(gt), loss, _ptr(yh))
        return np.array(loss[:], np.float64), yh

    def autotune(self):
        """After a forward: time the CRF tiles on the hinge's problem and enter the fastest in the
        process-wide tile table (no bit changes; synchronises)."""
        call("cnncrf_train_autotune", self._h)

    def hinge_grads(self):
        """Copies of the last hinge's subgradients (volume, pairwise output)."""
        v, p = C.c_void_p(), C.c_void_p()
        call("cnncrf_train_hinge_grads", self._h, C.byref(v), C.byref(p))
        return (as_device_tensor(v.value, (self.n, self.H, self.W, self.D)).clone(),
                as_device_tensor(p.value, (self.n, 2, self.H, self.W)).clone())

    def backward(self, gvol=None, gpw=None):
        """Gradients of sum(gvol * vol) + sum(gpw * pw), or of the hinge loss."""
        gv = None if gvol is None else gvol.contiguous()
        gp = None if gpw is None else gpw.contiguous()
        call("cnncrf_train_backward", self._h, None if gv is None else _ptr(gv), None if gp is None else _ptr(gp))

    def sgd(self, lr=1e-3, momentum=0.9):
        call("cnncrf_train_sgd", self._h, lr, momentum)

    def step(self, left, right, gt, lr=1e-3, momentum=0.9):
        loss = (C.c_double * self.n)()
        call("cnncrf_train_step", self._h, _ptr(left.contiguous()), _ptr(right.contiguous()), _ptr(gt.contiguous()),
             lr, momentum, loss)
        return np.array(loss[:], np.float64)


class StereoNetsFunction(torch.autograd.Function):
    """(left, right, *params) -> (unary volume, pairwise |h|) with the library's adjoints."""

    @staticmethod
    def forward(ctx, trainer, left, right, *params):
        for i, p in enumerate(params):
            trainer.set_param(i, p)
        vol, pw = trainer.forward(left, right)
        ctx.trainer = trainer
        ctx.nparams = len(params)
        return vol.clone(), pw.clone()

    @staticmethod
    def backward(ctx, gvol, gpw):
        t = ctx.trainer
        t.backward(gvol.float().contiguous(), gpw.float().contiguous())
        return (None, None, None) + tuple(t.grad_tensor(i) for i in range(ctx.nparams))


class HingeLossFunction(torch.autograd.Function):
    """The structured hinge of the batch: the mean of the pairs' per-pixel
    losses (mean_loss) or the sum of their losses.  vol and pw must be the
    trainer's last forward outputs: the CRF runs on its own copies of them."""

    @staticmethod
    def forward(ctx, trainer, vol, pw, gt):
        losses, _ = trainer.hinge(gt)
        ctx.trainer = trainer
        total = losses.mean() if trainer.mean_loss else losses.sum()
        return torch.tensor(float(total), dtype=torch.float64, device=vol.device)

    @staticmethod
    def backward(ctx, g):
        gvol, gpw = ctx.trainer.hinge_grads()
        s = g.float()
        return None, gvol * s, gpw * s, None
