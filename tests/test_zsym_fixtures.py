"""The complex symmetric fixtures, read against a dense model: upstream's
'S' product applies the Helmholtz matrix A, its 'H' product the Hermitian
matrix completed from A's UPLO triangle *in cluster numbering* with a real
diagonal (hemv / hemm on the diagonal leaves, op 'C' for the stored
off-diagonal leaves: hmatrix.hpp:843-911, matrix.hpp:386-447), both within
the compression error.  This pins what the GPU parity tests compare
against."""
import numpy as np
import pytest

NAMES = ["helmholtz_cube2000_zsymSU", "helmholtz_cube2000_zsymSL", "helmholtz_cube2000_zsymHU", "helmholtz_cube2000_zsymHL", "helmholtz_cube2000_zsymaca"]


@pytest.mark.parametrize("name", NAMES)
def test_zsym_fixture_semantics(port, golden, name):
    g, meta = golden(name)
    pts = g["xt"]
    n = pts.shape[0]
    perm = port.cluster(pts).export()[0]
    P = pts[perm]
    r = np.sqrt(((P[:, None, :] - P[None, :, :]) ** 2).sum(-1))
    with np.errstate(divide="ignore", invalid="ignore"):
        A = np.where(r == 0, 0.0, np.exp(1j * meta["wavenumber"] * r) / (4 * np.pi * r))  # cluster numbering
    if meta["symmetry"] == "H":
        T = np.tril(A, -1) if meta["uplo"] == "L" else np.triu(A, 1)
        A = T + T.conj().T + np.diag(A.diagonal().real)
    for mu in (1, 3):
        x = g["x_mu%d" % mu].reshape(mu, n).T[perm]
        for key, M in (("y_mu%d", A), ("yT_mu%d", A.T)):
            y = g[key % mu].reshape(mu, n).T[perm]
            assert np.linalg.norm(M @ x - y) / np.linalg.norm(y) < 10 * meta["eps"], (key, mu)
