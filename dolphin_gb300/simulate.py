"""Seeded synthetic SLC stacks for tests and benchmarks.

Follows the construction of the reference's simulator
(``src/dolphin/phase_link/simulate.py``): an exponential-decay coherence model
``Gamma_ij = (gamma0 - gamma_inf) * exp(-|t_i - t_j| / tau) + gamma_inf`` with a unit
diagonal (simulate.py:174,186-192), per-pixel amplitudes (the ``amplitudes``
argument, simulate.py:131,167-170), a Gaussian deformation bump growing linearly in
time (``make_defo_stack``, simulate.py:298-325) and circular-Gaussian samples drawn
through a Cholesky factor of the covariance (``make_noisy_samples``,
simulate.py:328-396).  Because ``diag(a) Gamma diag(a)`` is factored by
``diag(a) chol(Gamma)``, one Cholesky factor serves every pixel.

Unlike the reference (whose module-level generator is unseeded), every draw here
comes from ``numpy.random.default_rng(seed)`` (or a seeded ``torch.Generator``
for the on-device variant used by the large benchmark), so a stack is
reproducible from its seed.

Persistent scatterers get amplitude ``ps_amp * (1 + ps_amp_jitter * N(0, 1))``: an
exactly constant amplitude has dispersion 0, which the PS selector treats as "no
data" (ps.py:242-243), so a 1 % jitter keeps them detectable.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

__all__ = ["StackConfig", "coherence_model", "make_stack", "make_stack_torch"]


@dataclass(frozen=True)
class StackConfig:
    nslc: int = 10
    rows: int = 128
    cols: int = 128
    seed: int = 20261204
    gamma0: float = 0.7
    gamma_inf: float = 0.1
    tau: float = 36.0
    acq_interval: float = 12.0
    amp_sigma: float = 0.3
    defo_peak: float = 3.0
    ps_frac: float = 0.05
    ps_amp: float = 10.0
    ps_amp_jitter: float = 0.01
    ps_phase_std: float = 0.05
    # optional high-coherence disk (centred, radius disk_radius * max(rows, cols)) whose
    # pixels follow the model with gamma0 = disk_gamma0 instead
    disk_gamma0: float | None = None
    disk_radius: float = 0.125
    # optional outlier pixels: with probability outlier_frac * col / cols a pixel's
    # amplitudes follow LogNormal(0, outlier_sigma) instead (varies the SHP counts)
    outlier_frac: float = 0.0
    outlier_sigma: float = 1.0


def coherence_model(nslc, gamma0, gamma_inf, tau, acq_interval=12.0):
    """Exponential-decay coherence matrix with unit diagonal (float64)."""
    t = np.arange(nslc) * acq_interval
    dt = np.abs(t[:, None] - t[None, :])
    g = (gamma0 - gamma_inf) * np.exp(-dt / tau) + gamma_inf
    np.fill_diagonal(g, 1.0)
    return g


def _disk_mask(cfg, r0=0, r1=None):
    rows, cols = cfg.rows, cfg.cols
    r1 = rows if r1 is None else r1
    r = np.arange(r0, r1)[:, None] - rows / 2.0
    c = np.arange(cols)[None, :] - cols / 2.0
    return r * r + c * c <= (cfg.disk_radius * max(rows, cols)) ** 2


def _defo_phase(nslc, rows, cols, peak):
    r = np.arange(rows)[:, None] - rows // 2
    c = np.arange(cols)[None, :] - cols // 2
    sigma = max(rows, cols) / 8.0
    bump = np.exp(-(r * r + c * c) / (2.0 * sigma * sigma))
    bump *= peak / bump.max()
    frac = np.linspace(0.0, 1.0, nslc)[:, None, None]
    return bump[None] * frac  # (nslc, rows, cols)


def make_stack(cfg: StackConfig = StackConfig(), return_truth=False):
    """Return an (nslc, rows, cols) complex64 stack (and optionally its PS mask/phase)."""
    rng = np.random.default_rng(cfg.seed)
    n, rows, cols = cfg.nslc, cfg.rows, cfg.cols
    gamma = coherence_model(n, cfg.gamma0, cfg.gamma_inf, cfg.tau, cfg.acq_interval)
    L = np.linalg.cholesky(gamma)
    npx = rows * cols
    w = (rng.normal(scale=np.sqrt(0.5), size=(n, npx))
         + 1j * rng.normal(scale=np.sqrt(0.5), size=(n, npx)))
    x = (L @ w).reshape(n, rows, cols)
    if cfg.disk_gamma0 is not None:
        Ld = np.linalg.cholesky(coherence_model(n, cfg.disk_gamma0, cfg.gamma_inf, cfg.tau, cfg.acq_interval))
        disk = _disk_mask(cfg)
        x[:, disk] = (Ld @ w)[:, disk.ravel()]
    amp = rng.lognormal(mean=0.0, sigma=cfg.amp_sigma, size=(n, rows, cols))
    if cfg.outlier_frac > 0:
        prob = cfg.outlier_frac * np.arange(cols)[None, :] / cols
        out = rng.random((rows, cols)) < prob
        amp[:, out] = rng.lognormal(mean=0.0, sigma=cfg.outlier_sigma, size=(n, int(out.sum())))
    phi = _defo_phase(n, rows, cols, cfg.defo_peak)
    z = amp * np.exp(1j * phi) * x
    ps = rng.random((rows, cols)) < cfg.ps_frac
    nps = int(ps.sum())
    if nps:
        ps_amp = cfg.ps_amp * (1.0 + cfg.ps_amp_jitter * rng.normal(size=(n, nps)))
        ps_phase = phi[:, ps] + cfg.ps_phase_std * rng.normal(size=(n, nps))
        z[:, ps] = ps_amp * np.exp(1j * ps_phase)
    z = z.astype(np.complex64)
    if return_truth:
        return z, ps, phi.astype(np.float32)
    return z


def make_stack_torch(cfg: StackConfig, device="cuda", rows_chunk=1024):
    """Same model generated on the GPU with a seeded ``torch.Generator``.

    Statistically identical to :func:`make_stack` (the random streams differ).
    Used for the multi-GB benchmark stacks, which numpy would take minutes to draw.
    """
    import torch

    n, rows, cols = cfg.nslc, cfg.rows, cfg.cols
    g = torch.Generator(device=device)
    g.manual_seed(cfg.seed)
    gamma = coherence_model(n, cfg.gamma0, cfg.gamma_inf, cfg.tau, cfg.acq_interval)
    L = torch.tensor(np.linalg.cholesky(gamma), dtype=torch.float32, device=device)
    Lc = torch.complex(L, torch.zeros_like(L))
    if cfg.disk_gamma0 is not None:
        Ld = torch.tensor(np.linalg.cholesky(coherence_model(n, cfg.disk_gamma0, cfg.gamma_inf, cfg.tau,
                                                             cfg.acq_interval)), dtype=torch.float32, device=device)
        Ldc = torch.complex(Ld, torch.zeros_like(Ld))
    out = torch.empty((n, rows, cols), dtype=torch.complex64, device=device)
    phi_full = torch.tensor(_defo_phase(n, rows, cols, cfg.defo_peak), dtype=torch.float32, device=device)
    for r0 in range(0, rows, rows_chunk):
        r1 = min(rows, r0 + rows_chunk)
        npx = (r1 - r0) * cols
        w = torch.complex(
            torch.randn((n, npx), generator=g, device=device) * np.sqrt(0.5),
            torch.randn((n, npx), generator=g, device=device) * np.sqrt(0.5),
        )
        x = (Lc @ w).reshape(n, r1 - r0, cols)
        if cfg.disk_gamma0 is not None:
            disk = torch.tensor(_disk_mask(cfg, r0, r1), device=device)
            xd = (Ldc @ w).reshape(n, r1 - r0, cols)
            x = torch.where(disk[None], xd, x)
        amp = torch.exp(cfg.amp_sigma * torch.randn((n, r1 - r0, cols), generator=g, device=device))
        if cfg.outlier_frac > 0:
            prob = cfg.outlier_frac * torch.arange(cols, device=device)[None, :] / cols
            out_px = torch.rand((r1 - r0, cols), generator=g, device=device) < prob
            amp_o = torch.exp(cfg.outlier_sigma * torch.randn((n, r1 - r0, cols), generator=g, device=device))
            amp = torch.where(out_px[None], amp_o, amp)
        phi = phi_full[:, r0:r1]
        z = amp * torch.polar(torch.ones_like(phi), phi) * x
        ps = torch.rand((r1 - r0, cols), generator=g, device=device) < cfg.ps_frac
        ps_amp = cfg.ps_amp * (1.0 + cfg.ps_amp_jitter * torch.randn((n, r1 - r0, cols), generator=g, device=device))
        ps_phase = phi + cfg.ps_phase_std * torch.randn((n, r1 - r0, cols), generator=g, device=device)
        zps = torch.polar(ps_amp, ps_phase)
        out[:, r0:r1] = torch.where(ps[None], zps, z)
    return out
