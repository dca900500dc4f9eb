"""The closed-shell reduction behind ccsdt_upload_cholesky, checked on the CPU: the reference's
antisymmetrized spin-orbital blocks built from Cholesky vectors (exachem/cholesky/v2tensors.cpp:
67-70 v2ijab, 76-78 v2ijka, 84-86 v2iabc), read at the alpha / alpha-beta positions the
closed-shell gather takes, equal the spatial Coulomb contractions sum_Q L L that the device
builds."""
import numpy as np

O, V, Q = 3, 4, 5


def _spin_orbital(L):
    """Spin-orbital vectors from spatial L[p][q][Q] (p, q over o occupied then v virtual spatial
    orbitals): spin-orbital index (p, spin) -> spin * n + p; the vector is zero between spins."""
    n = L.shape[0]
    Lso = np.zeros((2 * n, 2 * n, L.shape[2]))
    Lso[:n, :n] = L
    Lso[n:, n:] = L
    return Lso


def test_reference_blocks_reduce_to_spatial_coulomb_integrals():
    rng = np.random.default_rng(7)
    n = O + V
    L = rng.normal(size=(n, n, Q))
    L = 0.5 * (L + L.transpose(1, 0, 2))
    Lso = _spin_orbital(L)
    occ = lambda i, s: s * n + i          # spin-orbital index of occupied i with spin s (0 alpha, 1 beta)
    vir = lambda a, s: s * n + O + a
    X = lambda p, q: Lso[p, q]             # cholVpr(p, q, Q) as a vector over Q
    oovv = np.empty((O, O, V, V))
    ooov = np.empty((O, O, O, V))
    ovvv = np.empty((O, V, V, V))
    for i in range(O):
        for j in range(O):
            for a in range(V):
                for b in range(V):
                    # v2ijab(h1, h2, p1, p2) = X(h1,p1).X(h2,p2) - X(h1,p2).X(h2,p1), read at (i_a, j_b, a_a, b_b)
                    h1, h2, p1, p2 = occ(i, 0), occ(j, 1), vir(a, 0), vir(b, 1)
                    oovv[i, j, a, b] = X(h1, p1) @ X(h2, p2) - X(h1, p2) @ X(h2, p1)
    for i in range(O):
        for j in range(O):
            for k in range(O):
                for a in range(V):
                    # v2ijka(h1, h2, h3, p1) = X(h1,h3).X(h2,p1) - X(h2,h3).X(h1,p1), read at (i_a, k_b, j_a, a_b)
                    h1, h2, h3, p1 = occ(i, 0), occ(k, 1), occ(j, 0), vir(a, 1)
                    ooov[i, j, k, a] = X(h1, h3) @ X(h2, p1) - X(h2, h3) @ X(h1, p1)
    for i in range(O):
        for a in range(V):
            for b in range(V):
                for c in range(V):
                    # v2iabc(h1, p1, p2, p3) = X(h1,p2).X(p1,p3) - X(h1,p3).X(p1,p2), read at (i_a, b_b, a_a, c_b)
                    h1, p1, p2, p3 = occ(i, 0), vir(b, 1), vir(a, 0), vir(c, 1)
                    ovvv[i, a, b, c] = X(h1, p2) @ X(p1, p3) - X(h1, p3) @ X(p1, p2)
    Loo, Lov, Lvv = L[:O, :O], L[:O, O:], L[O:, O:]
    np.testing.assert_allclose(oovv, np.einsum("iaQ,jbQ->ijab", Lov, Lov), rtol=0, atol=1e-12)
    np.testing.assert_allclose(ooov, np.einsum("ijQ,kaQ->ijka", Loo, Lov), rtol=0, atol=1e-12)
    np.testing.assert_allclose(ovvv, np.einsum("iaQ,bcQ->iabc", Lov, Lvv), rtol=0, atol=1e-12)
