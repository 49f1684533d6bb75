"""Differentiable three-phonon linewidths and kappa_sma with respect to the third-order
force constants, behind torch.autograd.Function.

Forward: tdg_set_fc3, tdg_scattering and tdg_kappa on the GB300 (ctypes). Backward: the
adjoint of get_kappa + symmetrize_kappa on the host (tdg_kappa_sma_vjp) and the adjoint
kernel (tdg_adjoint_fc3), which recomputes Psi per q-triplet instead of storing it.
Tensors are CPU float64, as the C-ABI takes host buffers; the work runs on the device.

Any parameterisation of Phi3 that is a torch function of parameters x composes with
ThreePhononKappa through autograd; fc3_from_irreducible is the symmetry-irreducible one
(Problem.fc3_irreducible, after the reference's forcemap).
"""
from __future__ import annotations

import numpy as np
import torch

from .scattering import Options, Problem, QLists, ScatteringRates

# Units of infile.forceconstant_thirdorder (eV/A^3) to Hartree/Bohr^3, and amu to electron
# masses (src/libolle/konstanter.f90).
FC3_EVA3_TO_AU = (1.0 / 27.21138602) * 0.52917721067 ** 3
AMU_TO_EMU = 1.660539040e-27 / 9.10938356e-31


def mass_weights(prob: Problem, masses_amu) -> np.ndarray:
    """1 / sqrt(m_i m_j m_k) of every third-order triplet ([n_fc3]) for atomic masses in amu:
    fc3_mwm = Phi3 [Hartree/Bohr^3] * mass_weights."""
    m = np.asarray(masses_amu, dtype=np.float64) * AMU_TO_EMU
    a = prob.fc3_atoms - 1
    return 1.0 / np.sqrt(m[a[:, 0]] * m[a[:, 1]] * m[a[:, 2]])


class ThreePhononKappa(torch.autograd.Function):
    """(fc3_mwm [n_fc3, 27]) -> (linewidth [n_irr, n_mode], kappa_sma [3, 3]), atomic units."""

    @staticmethod
    def forward(ctx, fc3_mwm: torch.Tensor, sr: ScatteringRates, opts: Options, lists: QLists):
        m = fc3_mwm.detach().to(torch.float64).cpu().numpy()
        sr.set_fc3(m)
        lw = sr.generate(opts, lists).copy()
        ks, _ = sr.kappa(opts, maxiter=0)
        ctx.sr, ctx.opts, ctx.lists = sr, opts, lists
        ctx.state = sr.linewidth
        ctx.save_for_backward(fc3_mwm.detach().clone())
        return torch.from_numpy(lw), torch.from_numpy(np.ascontiguousarray(ks))

    @staticmethod
    def backward(ctx, g_lw, g_ks):
        sr, opts, lists = ctx.sr, ctx.opts, ctx.lists
        (m,) = ctx.saved_tensors
        if sr.linewidth is not ctx.state:
            # another forward ran on this context since: restore this one's state
            sr.set_fc3(m.cpu().numpy())
            sr.generate(opts, lists)
        p = sr.prob
        lw_bar = np.zeros((p.n_irr, p.n_mode))
        if g_lw is not None:
            lw_bar += g_lw.detach().cpu().numpy()
        if g_ks is not None:
            lw_bar += sr.kappa_sma_vjp(opts, g_ks.detach().cpu().numpy())
        grad = sr.adjoint_fc3(opts, lw_bar)
        return torch.from_numpy(grad).to(m.dtype), None, None, None


def linewidth_and_kappa(fc3_mwm: torch.Tensor, sr: ScatteringRates, opts: Options, lists: QLists):
    """Differentiable (linewidth, kappa_sma) of the given mass-weighted Phi3."""
    return ThreePhononKappa.apply(fc3_mwm, sr, opts, lists)


def fc3_from_irreducible(x: torch.Tensor, B) -> torch.Tensor:
    """Mass-weighted Phi3 [n_fc3, 27] = B x for the symmetry-irreducible parameters x
    (Problem.fc3_irreducible returns x and the sparse B); differentiable in x, so
    d kappa / d x = B^T d kappa / d fc3_mwm comes out of autograd."""
    coo = B.tocoo()
    idx = torch.from_numpy(np.vstack([coo.row, coo.col]).astype(np.int64))
    Bt = torch.sparse_coo_tensor(idx, torch.from_numpy(coo.data), size=coo.shape, dtype=torch.float64)
    return torch.sparse.mm(Bt, x.reshape(-1, 1)).reshape(-1, 27)
