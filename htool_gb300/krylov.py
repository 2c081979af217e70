"""Krylov solves that apply the H-matrix as a replayed CUDA graph.

htool is driven by HPDDM in iterative use: HPDDM's GMV
(include/htool/wrappers/wrapper_hpddm.hpp:41-83) calls the product in local
numbering, mvprod_local_to_local (include/htool/types/hmatrix.hpp:1185-1274),
once per Krylov iteration.  Here the product is captured once on fixed
device buffers (an HBatch entry, optionally in cluster numbering) and every
application is one graph launch on the caller's stream; the Krylov vectors
live on the device.

GMRES(m) with classical Gram-Schmidt and one reorthogonalisation, Givens
rotations on the small Hessenberg matrix (host), restarts every m steps.
"""
import numpy as np

from . import CLUSTER_NUMBERING, HBatch


class GraphOperator:
    """y = H x for one right-hand side on fixed device buffers, captured as
    a CUDA graph; local=True works in cluster numbering (HPDDM's GMV)."""

    def __init__(self, hmatrix, local=False, device=0):
        import torch

        nr, nc, _, _ = hmatrix.sizes()
        self.shape = (nr, nc)
        self.hmatrix = hmatrix
        self.x = torch.zeros(nc, dtype=torch.float64, device="cuda:%d" % device)
        self.y = torch.zeros(nr, dtype=torch.float64, device="cuda:%d" % device)
        self.batch = HBatch(device)
        self.batch.add(hmatrix, self.x.data_ptr(), self.y.data_ptr(), 1, keep=(self.x, self.y), flags=CLUSTER_NUMBERING if local else 0)
        self.batch.capture(1)
        self.applications = 0

    def __call__(self, v):
        import torch

        self.x.copy_(v)
        self.batch.launch(torch.cuda.current_stream().cuda_stream)
        self.applications += 1
        return self.y.clone()


def gmres(op, b, x0=None, restart=40, tol=1e-10, maxiter=500):
    """Solve op(x) = b; b (and x0) torch vectors, op maps a vector to a new
    vector on the same device.  Returns (x, relative residual history): the
    true residual ||b - op(x)|| / ||b|| at every restart plus the Arnoldi
    estimate after every step."""
    import torch

    n = b.numel()
    x = torch.zeros_like(b) if x0 is None else x0.clone()
    bnorm = float(torch.linalg.norm(b))
    if bnorm == 0.0:
        return torch.zeros_like(b), [0.0]
    hist = []
    steps = 0
    while True:
        r = b - op(x)
        beta = float(torch.linalg.norm(r))
        hist.append(beta / bnorm)
        if beta / bnorm <= tol or steps >= maxiter:
            return x, hist
        m = min(restart, maxiter - steps)
        V = torch.empty((m + 1, n), dtype=b.dtype, device=b.device)
        V[0] = r / beta
        Hs = np.zeros((m + 1, m))
        cs, sn = np.zeros(m), np.zeros(m)
        g = np.zeros(m + 1)
        g[0] = beta
        k = 0
        for j in range(m):
            w = op(V[j])
            h = V[: j + 1] @ w
            w = w - V[: j + 1].T @ h
            h2 = V[: j + 1] @ w  # reorthogonalisation
            w = w - V[: j + 1].T @ h2
            hcol = (h + h2).cpu().numpy()
            hn = float(torch.linalg.norm(w))
            Hs[: j + 1, j] = hcol
            Hs[j + 1, j] = hn
            if hn > 0.0:
                V[j + 1] = w / hn
            for i in range(j):  # earlier rotations on the new column
                t = cs[i] * Hs[i, j] + sn[i] * Hs[i + 1, j]
                Hs[i + 1, j] = -sn[i] * Hs[i, j] + cs[i] * Hs[i + 1, j]
                Hs[i, j] = t
            den = np.hypot(Hs[j, j], Hs[j + 1, j])
            cs[j], sn[j] = (1.0, 0.0) if den == 0.0 else (Hs[j, j] / den, Hs[j + 1, j] / den)
            Hs[j, j] = cs[j] * Hs[j, j] + sn[j] * Hs[j + 1, j]
            Hs[j + 1, j] = 0.0
            g[j + 1] = -sn[j] * g[j]
            g[j] = cs[j] * g[j]
            k = j + 1
            steps += 1
            hist.append(abs(g[j + 1]) / bnorm)
            if abs(g[j + 1]) / bnorm <= tol or hn == 0.0:
                break
        # x += V_k y with the triangular solve of the rotated Hessenberg matrix
        y = np.zeros(k)
        for i in range(k - 1, -1, -1):
            y[i] = (g[i] - Hs[i, i + 1 : k] @ y[i + 1 : k]) / Hs[i, i]
        x = x + V[:k].T @ torch.from_numpy(y).to(device=b.device, dtype=b.dtype)
