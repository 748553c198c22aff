"""CPU FP64 oracle of the Nyström discretisation: test infrastructure.  Only tests/ and
bench.py's CPU-baseline leg import it, as the checker; the library never calls it.

Restates the reference's rigid/soft Nyström system on the surface quadrature nodes:

* operators S, D, K', H at the nodes with node weights and zero coincident entries, the
  Burton-Miller / CBIE combinations and right-hand sides of ``_assemble_full_boundary`` and
  ``_solve_full_boundary`` (solvers/bem/full.jl:68-128, 130-184);
* the density-interpolation correction in the structure of ``_fluid_layer_operators``
  (solvers/bem/quadrature/fluid.jl:94-163): the defect of the discrete Green identity
  ``mult * u + S du/dn - D u`` (and its normal-derivative form ``mult * du/dn + K' du/dn -
  H u``, ``mult = -1/2`` on the surface) on a basis of Helmholtz solutions, fitted per
  target on its nearest element (for on-surface targets, the target's own element) by a
  scaled minimum-norm solve through an SVD with the 1e-13 relative cutoff
  (fluid.jl:130-136); corrections ``S -= w_flux``, ``D += w_pressure`` (fluid.jl:137-139).

The basis is nine plane waves exp(i k d . y) with fixed integer directions (the general
correction of the reference lives in Inti.jl, a third-party package not present here; the
plane-wave basis is this build's choice, after the plane-wave density interpolation of
Perez-Arancibia, Faria and Turc 2019).  The far field is the node sum of full.jl:509-519.
"""
import math

import numpy as np

from . import oracle as O

# Radon 7-point rule weights (barycentric rule of the panel records)
RULE_W = np.array([0.225] + [0.13239415278850618] * 3 + [0.12593918054482715] * 3)
NODES = 7
_DIRS = np.array([(3, 1, -1), (-3, -2, 2), (-3, 1, -1), (1, 2, -3), (2, 2, 3), (0, 1, 2),
                  (0, -1, -1), (-1, -3, 1), (-3, -3, -1)], dtype=np.float64)


def directions():
    """The nine unit plane-wave directions (integer vectors over a rounded square root)."""
    a, b, c = _DIRS[:, 0], _DIRS[:, 1], _DIRS[:, 2]
    nr = np.sqrt(a * a + b * b + c * c)
    return np.stack([a / nr, b / nr, c / nr], axis=1)


def nodes_of(P: O.Panels):
    """Node positions (N x 3), element normals (N x 3) and weights (N), element-major."""
    y = P.gauss.reshape(-1, 3).copy()
    ny = np.repeat(P.normals, NODES, axis=0)
    w = (P.areas[:, None] * RULE_W[None, :]).reshape(-1)
    return y, ny, w


def operators(y, ny, w, k):
    """Weighted node operators S, D, K', H (N x N), zero on coincident nodes."""
    d = y[:, None, :] - y[None, :, :]
    r = np.sqrt((d * d).sum(-1))
    same = r == 0
    r = np.where(same, 1.0, r)
    ir = 1.0 / r
    G = np.exp(1j * k * r) * ir / (4 * np.pi)
    G1 = G * (1j * k - ir)
    G2 = G * ((1j * k - ir) ** 2 + ir ** 2)
    dny = (d * ny[None, :, :]).sum(-1)
    dnx = (d * ny[:, None, :]).sum(-1)
    nn = ny @ ny.T
    S = G * w[None, :]
    D = -G1 * dny * ir * w[None, :]
    K = G1 * dnx * ir * w[None, :]
    H = -((G2 - G1 * ir) * dnx * dny * ir * ir + G1 * nn * ir) * w[None, :]
    for A in (S, D, K, H):
        A[same] = 0
    return S, D, K, H


def traces(y, ny, k):
    """Plane-wave traces u (N x 9) and du/dn (N x 9) at the nodes."""
    dirs = directions()
    u = np.exp(1j * k * (y @ dirs.T))
    return u, 1j * k * (ny @ dirs.T) * u


def fit_weights(u, f, defect, cutoff=1e-13):
    """Per element: minimum-norm weights of the scaled trace fit (fluid.jl:130-136).

    Returns W (elements x 7 targets x 14 weights): pressure weights then flux weights."""
    N = u.shape[0]
    ne = N // NODES
    M = np.concatenate([u.reshape(ne, NODES, -1), f.reshape(ne, NODES, -1)], axis=1)
    sc = np.maximum(np.sqrt((np.abs(M) ** 2).sum(2)), np.finfo(float).eps)  # (ne, 14)
    A = np.transpose(M / sc[:, :, None], (0, 2, 1))  # (ne, 9, 14), plain transpose
    U, s, Vh = np.linalg.svd(A, full_matrices=False)
    keep = s > cutoff * s[:, :1]
    sinv = np.where(keep, 1.0 / np.where(keep, s, 1.0), 0.0)
    pinv = np.einsum("eij,ej,ekj->eik", np.conj(np.transpose(Vh, (0, 2, 1))), sinv, np.conj(U))
    dfx = defect.reshape(ne, NODES, -1)  # (ne, 7 targets, 9)
    W = np.einsum("eiq,etq->eti", pinv, dfx) / sc[:, None, :]
    return W, int((~keep).sum())


def corrected_operators(P: O.Panels, k):
    """S, D, K', H with the element corrections, and the nodes (y, ny, w)."""
    y, ny, w = nodes_of(P)
    S, D, K, H = operators(y, ny, w, k)
    u, f = traces(y, ny, k)
    def_sd = -0.5 * u + S @ f - D @ u
    def_kh = -0.5 * f + K @ f - H @ u
    W1, _ = fit_weights(u, f, def_sd)
    W2, _ = fit_weights(u, f, def_kh)
    ne = len(w) // NODES
    for e in range(ne):
        c = slice(e * NODES, (e + 1) * NODES)
        D[c, c] += W1[e][:, :NODES]
        S[c, c] -= W1[e][:, NODES:]
        H[c, c] += W2[e][:, :NODES]
        K[c, c] -= W2[e][:, NODES:]
    return (S, D, K, H), (y, ny, w)


def assemble(P: O.Panels, k, burton_miller=True):
    """M1 = 1/2 I - D - a H and M2 = S + a (1/2 I + K') on the nodes (a = i/k or 0)."""
    (S, D, K, H), _ = corrected_operators(P, k)
    a = 1j / k if burton_miller else 0.0
    I = np.eye(S.shape[0])
    return 0.5 * I - D - a * H, S + a * (0.5 * I + K)


def _element_pinv(u_e, f_e, cutoff=1e-13):
    """Pseudo-inverse (14 x 9) of one element's scaled trace fit and its row scales."""
    M = np.concatenate([u_e, f_e], axis=0)
    sc = np.maximum(np.sqrt((np.abs(M) ** 2).sum(1)), np.finfo(float).eps)
    A = (M / sc[:, None]).T
    U, s, Vh = np.linalg.svd(A, full_matrices=False)
    keep = s > cutoff * s[0]
    return (Vh[keep].conj().T / s[keep]) @ U[:, keep].conj().T, sc


def _inside(P: O.Panels, x):
    """Solid angle of the closed surface seen from x (Van Oosterom-Strackee) > 2 pi."""
    R = P.vertices - x[None, None, :]
    r = np.linalg.norm(R, axis=2)
    R0, R1, R2 = R[:, 0], R[:, 1], R[:, 2]
    num = np.einsum("ij,ij->i", R0, np.cross(R1, R2))
    den = (r[:, 0] * r[:, 1] * r[:, 2] + np.einsum("ij,ij->i", R0, R1) * r[:, 2] +
           np.einsum("ij,ij->i", R0, R2) * r[:, 1] + np.einsum("ij,ij->i", R1, R2) * r[:, 0])
    return 2.0 * np.arctan2(num, den).sum() > 2.0 * np.pi


def pressure(P: O.Panels, k, points, p, q, direction, field="scattered", g=None, h=None):
    """Field of a Nyström solution at points, in the reference's point-evaluation form
    (fields/pressure.jl:448-467 through quadrature/fluid.jl:94-163 with
    exclude_nearest=true): the element of the nearest node is left out of the node sum and
    its contribution recovered from the fit of the interpolants' defect
    mult u(x) + S_excl du/dn - D_excl u (mult 0 outside, -1 inside).  Outside:
    u_s = sum_j w_j (dG/dn_y p_j - G q_j); inside a fluid body (g, h given): the interior
    field sum_j w_j (G g (q + q_inc)_j - dG/dn_y (p + p_inc)_j) at k / h."""
    y, ny, w = nodes_of(P)
    fluid = g is not None
    d_inc = np.asarray(direction, dtype=np.float64)
    pin = np.exp(1j * k * (y @ d_inc))
    qin = 1j * k * (ny @ d_inc) * pin
    out = []
    for x in np.asarray(points, dtype=np.float64).reshape(-1, 3):
        inc = np.exp(1j * k * (x @ d_inc))
        if field == "incident":
            out.append(inc)
            continue
        inside = _inside(P, x)
        if inside and not fluid:
            raise ValueError("point lies inside the body")
        if (field == "interior") != inside and field != "total":
            raise ValueError("the field does not exist at this point")
        kk = k / h if inside else k
        u_all, f_all = traces(y, ny, kk)
        dp, dq = (p + pin, g * (q + qin)) if inside else (p, q)
        dv = x[None, :] - y
        r2 = (dv * dv).sum(1)
        b = (int(np.argmin(r2)) // NODES) * NODES
        keep = np.ones(len(w), dtype=bool)
        keep[b:b + NODES] = False
        r = np.sqrt(r2[keep])
        ir = 1.0 / r
        G = np.exp(1j * kk * r) * ir / (4 * np.pi)
        G1 = G * (1j * kk - ir)
        S = G * w[keep]
        D = -G1 * (dv[keep] * ny[keep]).sum(1) * ir * w[keep]
        sg = -1.0 if inside else 1.0
        fld = sg * np.sum(D * dp[keep] - S * dq[keep])
        defect = S @ f_all[keep] - D @ u_all[keep]
        if inside:
            defect = defect - np.exp(1j * kk * (directions() @ x))
        pinv, sc = _element_pinv(u_all[b:b + NODES], f_all[b:b + NODES])
        wt = (pinv @ defect) / sc
        fld += sg * (wt[:NODES] @ dp[b:b + NODES] + wt[NODES:] @ dq[b:b + NODES])
        out.append(fld + inc if (field == "total" and not inside) else fld)
    return np.array(out)


def assemble_fluid(P: O.Panels, k, g, h, formulation="muller"):
    """The fluid system on the nodes (full.jl:289-346 block algebra, as the panel oracle):
    Mueller [I - De + Di, Se - g Si; -He + Hi/g, I + K'e - K'i], CBIE [1/2 I - De, Se;
    1/2 I + Di, -g Si], each wavenumber's operators corrected by its own plane waves."""
    (Se, De, Ke, He), _ = corrected_operators(P, k)
    (Si, Di, Ki, Hi), _ = corrected_operators(P, k / h)
    I = np.eye(Se.shape[0])
    if formulation == "muller":
        return np.block([[I - De + Di, Se - g * Si], [-He + Hi / g, I + Ke - Ki]])
    return np.block([[0.5 * I - De, Se], [0.5 * I + Di, -g * Si]])


def far_field(y, ny, w, k, xhat, p, q):
    """f(xhat) = -(1/4 pi) sum_i w_i (i k xhat.n_i p_i + q_i) e^{-i k xhat.y_i}."""
    xhat = np.asarray(xhat, dtype=np.float64)
    return complex(-np.sum(w * (1j * k * (ny @ xhat) * p + q) *
                           np.exp(-1j * k * (y @ xhat))) / (4 * np.pi))


def solve(nodes, triangles, boundary, k, incidence_angle=math.pi / 2, incidence_azimuth=0.0,
          formulation=None, g=1.0, h=1.0):
    """Scattered traces at the nodes (full.jl:130-184 for rigid / pressure-release bodies,
    full.jl:422-495 for fluid ones, the direct solve in place of GMRES).
    Returns (p, q, (y, ny, w))."""
    P = O.Panels(nodes, triangles)
    d = O.incidence_direction(incidence_angle, incidence_azimuth)
    if boundary == "fluid":
        formulation = formulation or "muller"
        y, ny, w = nodes_of(P)
        n = len(w)
        pin = np.exp(1j * k * (y @ d))
        qin = 1j * k * (ny @ d) * pin
        A = assemble_fluid(P, k, g, h, formulation)
        if formulation == "muller":
            x = np.linalg.solve(A, np.concatenate([pin, qin]))
            return x[:n] - pin, x[n:] - qin, (y, ny, w)
        b = np.zeros(2 * n, dtype=np.complex128)
        b[n:] = -(A[n:, :] @ np.concatenate([pin, qin]))
        x = np.linalg.solve(A, b)
        return x[:n], x[n:], (y, ny, w)
    formulation = formulation or "burton_miller"
    (S, D, K, H), (y, ny, w) = corrected_operators(P, k)
    a = 1j / k if formulation == "burton_miller" else 0.0
    I = np.eye(len(w))
    pin = np.exp(1j * k * (y @ d))
    qin = 1j * k * (ny @ d) * pin
    if boundary == "rigid":
        A = 0.5 * I - D - a * H
        b = S @ qin + a * (0.5 * qin + K @ qin)
        p = np.linalg.solve(A, b)
        q = -qin
    else:
        A = S + a * (0.5 * I + K)
        b = -(D @ pin) + 0.5 * pin - a * (H @ pin)
        q = np.linalg.solve(A, b)
        p = -pin
    return p, q, (y, ny, w)


def neighbourhoods(y, count=48):
    """Element neighbourhoods of the restricted additive Schwarz preconditioner: for
    element e, the `count` elements whose centroids are nearest to e's (e itself first,
    ties by index).  y: node positions (element-major, 7 per element); an element's first
    node is the rule's centroid node."""
    ne = len(y) // NODES
    cent = y[::NODES]
    out = []
    idx = np.arange(ne)
    for e in range(ne):
        d = ((cent - cent[e]) ** 2).sum(1)
        order = np.lexsort((idx, d))
        out.append(order[:min(count, ne)])
    return out


def ras_matrix(A, nbhd):
    """Restricted additive Schwarz preconditioner P^-1 (dense N x N) of the node system A:
    for every element e, the rows of its own nodes of inv(A[N_e, N_e]), placed at the
    columns of N_e (the nodes of its neighbourhood's elements, in neighbourhood order)."""
    n = A.shape[0]
    Pinv = np.zeros((n, n), dtype=np.complex128)
    for e, els in enumerate(nbhd):
        idx = (els[:, None] * NODES + np.arange(NODES)[None, :]).reshape(-1)
        inv = np.linalg.inv(A[np.ix_(idx, idx)])
        Pinv[e * NODES:(e + 1) * NODES, idx] = inv[:NODES, :]   # e is the first element
    return Pinv


def assemble_regions(surfaces, materials, parents, k, formulation="muller"):
    """Coupled fluid regions on the quadrature nodes: the block algebra of the panel
    oracle's ``assemble_regions`` (solvers/bem/regions.jl:189-236) with node operators.
    Surface i (1-based) encloses region i, parents[i-1] is the region outside it, materials
    (density, sound speed) per region relative to the exterior.  Between different surfaces
    the operators are the plain node kernel at the region's wavenumber; a surface's own
    block at the wavenumber of each region it borders is ``corrected_operators`` of that
    surface alone (the Green identities hold surface by surface).
    Returns (A, (y, ny, w) of all nodes in surface order, node offsets)."""
    Ps = [O.Panels(nd, tr) for nd, tr in surfaces]
    per = [nodes_of(P) for P in Ps]
    y = np.concatenate([p[0] for p in per])
    ny = np.concatenate([p[1] for p in per])
    w = np.concatenate([p[2] for p in per])
    offs = [0]
    for p in per:
        offs.append(offs[-1] + len(p[2]))
    n = offs[-1]
    count = len(surfaces)
    dens = [1.0] + [float(m[0]) for m in materials]
    speeds = [1.0] + [float(m[1]) for m in materials]
    ops = {}

    def region_ops(r):
        if r not in ops:
            kr = k / speeds[r]
            S, D, K, H = operators(y, ny, w, kr)
            for s in range(1, count + 1):
                if not (s == r or parents[s - 1] == r):
                    continue
                blk = slice(offs[s - 1], offs[s])
                (Ss, Ds, Ks, Hs), _ = corrected_operators(Ps[s - 1], kr)
                S[blk, blk], D[blk, blk], K[blk, blk], H[blk, blk] = Ss, Ds, Ks, Hs
            ops[r] = (S, D, K, H)
        return ops[r]

    A = np.eye(2 * n, dtype=np.complex128) if formulation == "muller" else \
        np.zeros((2 * n, 2 * n), dtype=np.complex128)
    for i in range(1, count + 1):
        rows = np.arange(offs[i - 1], offs[i])
        for region in (i, parents[i - 1]):
            rho = dens[region]
            S, D, K, H = region_ops(region)
            eqs = rows + n if region == i else rows
            if formulation == "cbie":
                A[np.ix_(eqs, rows)] += 0.5 * np.eye(len(rows))
            for j in range(1, count + 1):
                if not (j == region or parents[j - 1] == region):
                    continue
                sign = 1.0 if j == region else -1.0
                cols = np.arange(offs[j - 1], offs[j])
                blk = np.ix_(rows, cols)
                if formulation == "cbie":
                    A[np.ix_(eqs, cols)] += sign * D[blk]
                    A[np.ix_(eqs, cols + n)] -= sign * rho * S[blk]
                    continue
                A[np.ix_(rows, cols)] += sign * D[blk]
                A[np.ix_(rows, cols + n)] -= sign * rho * S[blk]
                A[np.ix_(rows + n, cols)] += (sign / rho) * H[blk]
                A[np.ix_(rows + n, cols + n)] -= sign * K[blk]
    return A, (y, ny, w), offs


def solve_regions(surfaces, materials, parents, k, incidence_angle=math.pi / 2,
                  incidence_azimuth=0.0, formulation="muller"):
    """Dense FP64 solve of the node region system with the plane wave on the surfaces that
    border the exterior (regions.jl:240-253) and the backscatter summed over them
    (solvers/bem/postprocessing.jl:15-31)."""
    A, (y, ny, w), offs = assemble_regions(surfaces, materials, parents, k, formulation)
    n = len(w)
    d = O.incidence_direction(incidence_angle, incidence_azimuth)
    pin = np.exp(1j * k * (y @ d))
    qin = 1j * k * (ny @ d) * pin
    outer = np.zeros(n, dtype=bool)
    b = np.zeros(2 * n, dtype=np.complex128)
    for i in range(1, len(surfaces) + 1):
        if parents[i - 1] == 0:
            sl = slice(offs[i - 1], offs[i])
            outer[sl] = True
            b[sl] = pin[sl]
            if formulation == "muller":
                b[n + offs[i - 1]:n + offs[i]] = qin[sl]
    x = np.linalg.solve(A, b)
    p_tot, v = x[:n], x[n:]
    ps = np.where(outer, p_tot - pin, 0.0)
    qs = np.where(outer, v - qin, 0.0)
    amp = far_field(y, ny, w, k, -d, ps, qs)
    return dict(A=A, b=b, x=x, amplitude=amp, p_scat=ps, dpdn_scat=qs, nodes=(y, ny, w),
                offsets=offs)
