"""Set-up linear algebra of the reference's linalg_utils.py that the differentiation
pattern needs: the modified (pivoted, truncated) Cholesky decomposition that
sampler.propagate_phaseless_ad_1 uses to rebuild the Cholesky vectors from a two-body
operator. torch FP64 on the device, differentiable (the pivots are chosen from the values,
as the reference's argmax does)."""

from __future__ import annotations

import torch


def modified_cholesky(mat: torch.Tensor, norb: int, nchol_max: int) -> torch.Tensor:
    """[nchol_max, size] vectors L with mat ~ sum_g L_g L_g^T (linalg_utils.py:70-106): the
    first pivot is the largest diagonal element, each next one the largest |residual
    diagonal|, L_{x+1} = (mat[nu] - sum_r L_r[nu] L_r) / sqrt(|residual[nu]|)."""
    diag = torch.diagonal(mat)
    nu = int(torch.argmax(diag).item())
    vecs = [mat[nu] / torch.sqrt(diag[nu])]
    approx = torch.zeros_like(diag)
    for x in range(nchol_max - 1):
        approx = approx + vecs[x] * vecs[x]
        delta = diag - approx
        nu = int(torch.argmax(torch.abs(delta)).item())
        r = vecs[0][nu] * vecs[0]
        for v in vecs[1:]:
            r = r + v[nu] * v
        vecs.append((mat[nu] - r) / torch.sqrt(torch.abs(delta[nu])))
    return torch.stack(vecs)
