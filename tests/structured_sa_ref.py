"""A numpy / scipy statement of the structured smoothed-aggregation hierarchy and its
V-cycle (cuibm_gb300/csrc/structured.cuh and the structured set-up in amg.cu), the
checker of the GPU's CUIBM_OP_PRECONDITION_POISSON.  Test infrastructure only.

Aggregates are 3 x 3 blocks of the level's grid (the last one along an axis takes
the remainder, cn = max(1, n // 3) per axis); the tentative prolongator is piecewise
constant with entries 1; P = (I - w D^-1 A) T with w = 4 / (3 rho(D^-1 A)), rho from
20 power iterations from the start vector 1 + 0.25 sin(0.37 i); A_c = P^T A P;
coarsening stops at or below KCOARSE unknowns, where the cycle inverts the level's
matrix.  The cycle: x = w D^-1 b, r = b - A x, b_c = P^T r down; x += P x_c, out =
x + w D^-1 (b - A x) up."""
import numpy as np
import scipy.sparse as sp

KCOARSE = 1500
POWER_ITERATIONS = 20


def coarse(n):
    return max(1, n // 3)


def axis_aggregates(n):
    cn = coarse(n)
    return np.minimum(np.arange(n) // 3, cn - 1), cn


def tentative(nx, ny):
    ax, cnx = axis_aggregates(nx)
    ay, cny = axis_aggregates(ny)
    agg = (ay[:, None] * cnx + ax[None, :]).ravel()
    n = nx * ny
    return sp.csr_matrix((np.ones(n), (np.arange(n), agg)), shape=(n, cnx * cny)), cnx, cny


def rho_dinv_a(A, dinv):
    n = A.shape[0]
    x = 1.0 + 0.25 * np.sin(0.37 * np.arange(n))
    x /= np.linalg.norm(x)
    s = 0.0
    for _ in range(POWER_ITERATIONS):
        y = dinv * (A @ x)
        s = float(np.dot(y, y))
        x = y / np.sqrt(s)
    return np.sqrt(s)


def hierarchy(A, nx, ny):
    """The levels of the structured hierarchy of the nx x ny operator A (CSR)."""
    levels = []
    A = sp.csr_matrix(A)
    while True:
        d = A.diagonal().copy()
        d[d == 0] = 1.0
        L = {"A": A, "dinv": 1.0 / d, "nx": nx, "ny": ny}
        levels.append(L)
        if len(levels) > 1 and A.shape[0] <= KCOARSE:
            L["inv"] = np.linalg.inv(A.toarray())
            return levels
        omega = 4.0 / (3.0 * rho_dinv_a(A, L["dinv"]))
        T, cnx, cny = tentative(nx, ny)
        P = (T - sp.diags(omega * L["dinv"]) @ (A @ T)).tocsr()
        L.update(omega=omega, P=P, R=P.T.tocsr())
        A = (P.T @ (A @ P)).tocsr()
        A.eliminate_zeros()
        nx, ny = cnx, cny


def vcycle(levels, b):
    bs, xs = [np.asarray(b, dtype=np.float64)], []
    for L in levels[:-1]:
        x = L["omega"] * L["dinv"] * bs[-1]
        xs.append(x)
        bs.append(L["R"] @ (bs[-1] - L["A"] @ x))
    xc = levels[-1]["inv"] @ bs[-1]
    for l in range(len(levels) - 2, -1, -1):
        L = levels[l]
        x = xs[l] + L["P"] @ xc
        xc = x + L["omega"] * L["dinv"] * (bs[l] - L["A"] @ x)
    return xc


def stencil_offsets(A, nx, ny):
    """The set of (dx, dy) grid offsets between a row and its columns in A."""
    C = sp.coo_matrix(A)
    dx = C.col % nx - C.row % nx
    dy = C.col // nx - C.row // nx
    return set(zip(dx.tolist(), dy.tolist()))
