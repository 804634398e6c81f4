"""Learned EMI warm start (no counterpart in the reference).

EMI finds the eigenvector of |Gamma|^-1 o C by inverse iteration from a constant
vector (phase_link/_eigenvalues.py:139-205).  ``WarmStartMLP`` reads a pixel's
coherence magnitudes (the N(N-1)/2 lower |C_ij|) and proposes the starting vector:
a fully connected network (ReLU on the hidden layers; 190 -> 256 -> 256 -> 40 at
N=20) trained on EMI solutions of the plain method.  Magnitudes carry no phase, so
the network's output is expressed in the frame of the pixel's own phases (those of
C_j0, each SLC's interferogram with SLC 0): the data supply the phases, the network
the rest.  Every step -- features, forward,
backward, Adam -- runs in the library's own kernels (``dpl_mlp_features``,
``dpl_gemm_f32``, ``dpl_relu_grad``, ``dpl_mse_grad``, ``dpl_colsum``, ``dpl_adam``);
torch only holds the device buffers.

``process_coherence_warm`` runs the solver with the network's vectors as starting
points.  Plain EMI stays the fallback: a pixel whose warm-started iteration does not
meet the stopping rule is iterated again from the constant vector, and the iteration
counts are returned so that the saving can be measured.
"""

from __future__ import annotations

import math

import numpy as np

from . import _device as D
from . import _lib

__all__ = ["WarmStartMLP", "make_training_set", "process_coherence_warm"]


def _check(st, what):
    _lib.check(st, what)


def _frame(C, V, conj_frame):
    """V (npix, N) complex rotated into (conj_frame=0) or out of (1) the phase frame of C."""
    torch = D.require_cuda()
    npix, n = V.shape
    out = torch.empty_like(V)
    _check(_lib.load().dpl_mlp_frame(D.ptr(C), int(n), npix, D.ptr(V), int(conj_frame), D.ptr(out),
                                     D.stream_handle()), "dpl_mlp_frame")
    return out


def _features(C, nslc, layout=1):
    """|C_ij| of the lower pairs: (npix, N(N-1)/2) float32 from (npix, N, N) complex64
    (layout 1) or planar (npix, N^2) float32 (layout 0) coherence."""
    torch = D.require_cuda()
    npix = C.shape[0]
    X = torch.empty((npix, nslc * (nslc - 1) // 2), dtype=torch.float32, device=C.device)
    _check(_lib.load().dpl_mlp_features(D.ptr(C), int(nslc), npix, int(layout), D.ptr(X), D.stream_handle()),
           "dpl_mlp_features")
    return X


class WarmStartMLP:
    """Fully connected network: nf -> hidden... -> 2N (re, im of the start vector)."""

    def __init__(self, nslc: int, hidden=(256, 256), seed: int = 0):
        torch = D.require_cuda()
        self.nslc = int(nslc)
        self.nf = self.nslc * (self.nslc - 1) // 2
        self.sizes = [self.nf, *[int(h) for h in hidden], 2 * self.nslc]
        rng = np.random.default_rng(seed)
        self.W, self.b = [], []
        for a, b in zip(self.sizes[:-1], self.sizes[1:]):
            w = rng.normal(scale=math.sqrt(2.0 / a), size=(b, a)).astype(np.float32)  # He initialisation
            self.W.append(torch.from_numpy(w).cuda())
            self.b.append(torch.zeros(b, dtype=torch.float32, device="cuda"))
        self._adam = None
        self._packed = None  # bf16 tensor-core copies of the weights (rebuilt after a change)
        self.step = 0

    # ---- plumbing -------------------------------------------------------------------
    @staticmethod
    def _gemm(M, N, K, A, sai, sak, B, sbj, sbk, C, sci, bias=None, alpha=1.0, beta=0.0, relu=False):
        lib = _lib.load()
        _check(lib.dpl_gemm_f32(M, N, K, D.ptr(A), sai, sak, D.ptr(B), sbj, sbk, D.ptr(C), sci, D.ptr(bias),
                                float(alpha), float(beta), int(relu), D.stream_handle()), "dpl_gemm_f32")

    def forward(self, X):
        """Layer outputs [H_1, ..., Y] for X (npix, nf) float32 on the device."""
        torch = D.require_cuda()
        outs = []
        h = X
        for k, (W, b) in enumerate(zip(self.W, self.b)):
            m, kin = h.shape
            nout = W.shape[0]
            out = torch.empty((m, nout), dtype=torch.float32, device=h.device)
            self._gemm(m, nout, kin, h, kin, 1, W, kin, 1, out, nout, bias=b, relu=k < len(self.W) - 1)
            outs.append(out)
            h = out
        return outs

    def tensor_core_ok(self) -> bool:
        """The tensor-core forward needs two hidden layers and widths of at most 256."""
        return len(self.W) == 3 and max(self.sizes) <= 256

    def forward_tc(self, X):
        """Network output Y (npix, 2N) float32 on the tensor cores (bf16 operands, fp32
        accumulation): inference only."""
        torch = D.require_cuda()
        lib = _lib.load()
        if not self.tensor_core_ok():
            raise ValueError("the tensor-core forward needs two hidden layers of width <= 256")
        if self._packed is None:
            packed = []
            for W in self.W:
                nout, nin = W.shape
                buf = torch.empty(int(lib.dpl_mlp_packed_bytes(nout, nin)), dtype=torch.uint8, device=W.device)
                _check(lib.dpl_mlp_pack(D.ptr(W.contiguous()), nout, nin, D.ptr(buf), D.stream_handle()),
                       "dpl_mlp_pack")
                packed.append(buf)
            self._packed = packed
        X = X.contiguous()
        npix = X.shape[0]
        Y = torch.empty((npix, self.sizes[-1]), dtype=torch.float32, device=X.device)
        status = torch.zeros(1, dtype=torch.int32, device=X.device)
        s = self.sizes
        _check(lib.dpl_mlp_forward_tc(D.ptr(X), npix, s[0], s[1], s[2], s[3], D.ptr(self._packed[0]), D.ptr(self.b[0]),
                                      D.ptr(self._packed[1]), D.ptr(self.b[1]), D.ptr(self._packed[2]),
                                      D.ptr(self.b[2]), D.ptr(Y), D.ptr(status), D.stream_handle()),
               "dpl_mlp_forward_tc")
        if int(status.item()) != 0:
            _check(int(status.item()), "dpl_mlp_forward_tc")
        return Y

    def gradients(self, X, T):
        """(loss parts, [(dW_l, db_l)]) of the mean squared error of forward(X) against T."""
        torch = D.require_cuda()
        lib = _lib.load()
        outs = self.forward(X)
        Y = outs[-1]
        count = Y.numel()
        dY = torch.empty_like(Y)
        parts = torch.empty((count + 255) // 256, dtype=torch.float32, device=Y.device)
        _check(lib.dpl_mse_grad(D.ptr(Y), D.ptr(T), D.ptr(dY), count, D.ptr(parts), D.stream_handle()),
               "dpl_mse_grad")
        grads = [None] * len(self.W)
        d = dY
        for k in range(len(self.W) - 1, -1, -1):
            h_in = X if k == 0 else outs[k - 1]
            m, kin = h_in.shape
            nout = self.W[k].shape[0]
            gW = torch.empty_like(self.W[k])
            # dW[j, i] = sum_r d[r, j] h_in[r, i]: op(A) = d^T (j, r), op(B) = h_in^T (i, r)
            self._gemm(nout, kin, m, d, 1, nout, h_in, 1, kin, gW, kin)
            gb = torch.empty_like(self.b[k])
            _check(lib.dpl_colsum(D.ptr(d), m, nout, D.ptr(gb), D.stream_handle()), "dpl_colsum")
            grads[k] = (gW, gb)
            if k > 0:
                dh = torch.empty_like(outs[k - 1])
                # dh[r, i] = sum_j d[r, j] W[j, i]: op(B) = W^T (i, j)
                self._gemm(m, kin, nout, d, nout, 1, self.W[k], 1, kin, dh, kin)
                _check(lib.dpl_relu_grad(D.ptr(outs[k - 1]), D.ptr(dh), dh.numel(), D.stream_handle()),
                       "dpl_relu_grad")
                d = dh
        return parts, count, grads

    def train_step(self, X, T, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        """One Adam step on the mean squared error; returns the loss (a host float)."""
        torch = D.require_cuda()
        lib = _lib.load()
        parts, count, grads = self.gradients(X, T)
        if self._adam is None:
            self._adam = [(torch.zeros_like(p), torch.zeros_like(p)) for pair in zip(self.W, self.b) for p in pair]
        self.step += 1
        self._packed = None
        params = [p for pair in zip(self.W, self.b) for p in pair]
        gradl = [g for pair in grads for g in pair]
        for p, g, (m1, m2) in zip(params, gradl, self._adam):
            _check(lib.dpl_adam(D.ptr(p), D.ptr(g), D.ptr(m1), D.ptr(m2), p.numel(), float(lr), float(b1), float(b2),
                                float(eps), self.step, D.stream_handle()), "dpl_adam")
        return float(parts.sum().item()) / count

    def features(self, C, layout=1):
        """Network input from coherence matrices: layout 1 = (npix, N, N) complex64."""
        return _features(C, self.nslc, layout)

    def predict(self, C, tensor_cores: bool = True):
        """Starting vectors (npix, N) complex64 for (npix, N, N) coherence matrices C: the
        network's output (on the tensor cores where the shape allows), in the frame of
        C's phases relative to SLC 0."""
        X = self.features(C, 1)
        Y = self.forward_tc(X) if tensor_cores and self.tensor_core_ok() else self.forward(X)[-1]
        return _frame(C, D.torch().view_as_complex(Y.view(-1, self.nslc, 2).contiguous()), 0)

    def state(self):
        return {f"W{k}": w.cpu().numpy() for k, w in enumerate(self.W)} | {
            f"b{k}": b.cpu().numpy() for k, b in enumerate(self.b)}

    def load_state(self, state):
        torch = D.require_cuda()
        self.W = [torch.from_numpy(np.asarray(state[f"W{k}"], np.float32)).cuda() for k in range(len(self.W))]
        self.b = [torch.from_numpy(np.asarray(state[f"b{k}"], np.float32)).cuda() for k in range(len(self.b))]
        self._adam, self.step, self._packed = None, 0, None


def make_training_set(npix_target, nslc=20, half_window=(5, 11), tile=64, seed=20261300):
    """Coherence matrices and their EMI solutions (plain method) for training.

    Tiles of ``tile x tile`` output pixels, each from its own seeded stack with
    gamma0 ~ U[0.3, 0.95], gamma_inf ~ U[0, 0.3], tau ~ U[12, 120] days.  Returns
    (X features (npix, nf), T targets (npix, 2N): the unit-norm EMI vector referenced to
    SLC 0 and expressed in the frame of C's phases relative to SLC 0), float32 on the
    device.
    """
    torch = D.require_cuda()
    from .phase_link import estimate_stack_covariance, process_coherence_matrices
    from .simulate import StackConfig, make_stack_torch

    rng = np.random.default_rng(seed)
    hy, hx = half_window
    feats, targs = [], []
    got, k = 0, 0
    while got < npix_target:
        g0 = rng.uniform(0.3, 0.95)
        cfg = StackConfig(nslc=nslc, rows=tile + 2 * hy, cols=tile + 2 * hx, seed=seed + 1 + k, gamma0=g0,
                          gamma_inf=rng.uniform(0.0, min(0.3, g0)), tau=rng.uniform(12.0, 120.0), ps_frac=0.0)
        z = make_stack_torch(cfg)
        C = estimate_stack_covariance(z, half_window)[hy:hy + tile, hx:hx + tile].reshape(-1, nslc, nslc)
        C = C.contiguous()
        v, _val, est, _crlb = process_coherence_matrices(C, compute_crlb=False)
        keep = (est == 1) & torch.isfinite(torch.view_as_real(v)).all(-1).all(-1)
        Ck = C[keep].contiguous()
        v = _frame(Ck, (v[keep] / math.sqrt(nslc)).contiguous(), 1)  # into the frame of C's phases
        feats.append(_features(Ck, nslc))
        targs.append(torch.view_as_real(v).reshape(v.shape[0], 2 * nslc).contiguous())
        got += int(keep.sum().item())
        k += 1
    return torch.cat(feats)[:npix_target].contiguous(), torch.cat(targs)[:npix_target].contiguous()


def process_coherence_warm(C, model=None, num_looks=1.0, compute_crlb=False, vstart=None):
    """EMI on (npix, N, N) complex64 CUDA coherence matrices, warm-started by `model`
    (or by explicit `vstart` vectors); returns (eigvecs, eigvals, estimator, crlb,
    temp_coh, iterations) as CUDA tensors."""
    torch = D.require_cuda()
    npix, n, _ = C.shape
    Cd = C.contiguous()
    if vstart is None and model is not None:
        vstart = model.predict(Cd)
    vec = torch.empty((npix, n), dtype=torch.complex64, device=Cd.device)
    val = torch.empty(npix, dtype=torch.float32, device=Cd.device)
    est = torch.empty(npix, dtype=torch.uint8, device=Cd.device)
    crlb = torch.empty((npix, n), dtype=torch.float32, device=Cd.device)
    tc = torch.empty(npix, dtype=torch.float32, device=Cd.device)
    clos = torch.empty((npix, max(n - 2, 1)), dtype=torch.float32, device=Cd.device)
    its = torch.empty(npix, dtype=torch.int16, device=Cd.device)
    lib = _lib.load()
    ws = D.workspace(lib.dpl_process_coherence_workspace_size(npix))
    _check(lib.dpl_process_coherence_warm(D.ptr(Cd), npix, n, 0, 0.0, 0.0, 0, float(num_looks), 0,
                                          int(bool(compute_crlb)), D.ptr(vstart), D.ptr(vec), D.ptr(val), D.ptr(est),
                                          D.ptr(crlb), D.ptr(tc), D.ptr(clos) if n > 2 else None, D.ptr(its),
                                          D.ptr(ws), ws.numel(), D.stream_handle()), "dpl_process_coherence_warm")
    return vec, val, est, crlb, tc, its
