"""Algorithmic work of the ADER-WENO step: FP64 flops and HBM bytes per unit.

The counts follow the reference algorithm (haranjackson/PyPDE src/), not
this implementation: they are what `roofline.achieved` divides by kernel
time.  Flops count +, -, *, / and sqrt as one each; a callback counts the
operations of its formula (F_FLOPS); max|eig| counts the nominal 10 m^3 of
a Hessenberg reduction plus Francis QR of the m x m block that carries the
spectrum: m = V, or the active block of a system whose passive variables
have zero rows and columns (their eigenvalues are isolated by a
permutation, exactly, as in LAPACK's balancing).

Units:
  face point   one (face, time node, transverse node) of fv.cpp:144-196
  w-cell       one cell of the reconstruction grid (n+2)^d
  cell-update  one interior cell advanced by one step
"""

# flops of one callback evaluation, counted from the formulas of
# pypde_gb300/csrc/systems.cuh (identical to the test callbacks)
def f_flops(system, ndim):
    if system == "euler":
        return 3 * ndim + 8
    if system == "cattaneo":
        return 3 * ndim + 8 + 3  # Euler part + T = p/rho, energy += q_d, kappa_h T
    if system == "ncp":
        return 8
    if system == "burgers2":
        return 5
    raise ValueError(system)


def b_flops(system):
    return 4 if system == "ncp" else 0


def s_flops(system, ndim):
    # cattaneo: 10^-x (Horner, degree 16: 32 + 4) and -q_i / tau
    return {"cattaneo": 36 + ndim, "ncp": 4}.get(system, 0)


def eig_flops(V):
    return 10 * V ** 3


def eig_active(system, ndim, V):
    """Size of the block of the flux Jacobian that carries its spectrum:
    cattaneo transports rho, the momenta, E and q_d in direction d; the
    other heat-flux components and log tau are passive."""
    return ndim + 3 if system == "cattaneo" else V


def max_abs_eigs_flops(system, ndim, V):
    """FD Jacobian (V+1 callbacks, V columns of V differences and V
    divisions, step h) + B + max|eig| of the active block
    (src/eigs/system.cpp:6-51)."""
    jac = (V + 1) * f_flops(system, ndim) + V * (2 + 2 * V)
    return jac + (V * V if b_flops(system) else 0) + eig_flops(eig_active(system, ndim, V))


def face_point_flops(system, ndim, V, N):
    """k_faces: endpoints, Rusanov flux, B path integral, weights, outputs."""
    ends = 2 * V * 2 * N
    rus = 2 * max_abs_eigs_flops(system, ndim, V) + 2 * V + 2 * f_flops(system, ndim) + 2 * V
    bint = N * (2 * V + b_flops(system) + 2 * V * V) + 2 * V * V + V if b_flops(system) else 0
    return ends + rus + bint + 3 + (ndim - 1) + 4 * V


def face_points(nX, N):
    ndim = len(nX)
    total = 0
    for d in range(ndim):
        nf = nX[d] + 1
        for e in range(ndim):
            if e != d:
                nf *= nX[e]
        total += nf * N * N ** (ndim - 1)
    return total


def weno_flops_per_output(N):
    """One 1-D reconstruction (N nodal values of one variable)."""
    nst = 2 if N <= 2 else (4 if N % 2 == 0 else 3)
    per_stencil = 2 * N * N + 2 * N * N + 1 + 3 + 1 + 2 * N + 1
    return nst * per_stencil + N


def cfl_flops_per_wcell(system, ndim, V, N):
    Nd = N ** ndim
    avg = V * 2 * Nd
    grads = ndim * V * (Nd * (2 * N + 1) + 2 * Nd)
    return avg + grads + ndim * (max_abs_eigs_flops(system, ndim, V) + 2)


def predictor_flops_per_iteration(system, ndim, V, N):
    """One Picard iteration of one cell (dg.cpp:50-126, 192-199)."""
    Nd = N ** ndim
    nodes = N * Nd
    per_node = (ndim * V * (2 * N + 1) + ndim * f_flops(system, ndim)
                + ndim * V * (2 * N + 1) + s_flops(system, ndim)
                + ndim * (V + (2 * V * V + b_flops(system) if b_flops(system) else 0))
                + 3 * V + V * (2 * N + 1) + 3 * V)
    return nodes * per_node


def newton_flops_per_iteration(system, ndim, V, N):
    """One Newton iteration of one cell (stiff predictor): the residual
    (as a Picard iteration), the FD Jacobian of S at every space-time node
    (V+1 S calls, V^2 differences and scalings), and per spatial node a
    dense LU of the (N V)^2 system (2/3 (NV)^3) and its solve (2 (NV)^2),
    counted dense and refreshed every iteration (the nominal cost)."""
    Nd = N ** ndim
    nl = N * V
    jac = N * Nd * ((V + 1) * s_flops(system, ndim) + 3 * V * V)
    lin = Nd * (2 * nl ** 3 // 3 + 2 * nl * nl)
    return predictor_flops_per_iteration(system, ndim, V, N) + jac + lin


def step_flops(system, nX, V, N, pred_iters_per_cell, stiff=False):
    """Whole-step algorithmic flops, per stage."""
    ndim = len(nX)
    C = 1
    Cw = 1
    for n in nX:
        C *= n
        Cw *= n + 2
    out = {}
    # WENO: pass d produces (cells of that pass) x N^d nodes x V outputs
    shape = [n + 2 * N for n in nX]
    weno = 0
    n4 = 1
    for d in range(ndim):
        shape[d] -= 2 * (N - 1)
        cells = 1
        for m in shape:
            cells *= m
        weno += cells * n4 * V * weno_flops_per_output(N)
        n4 *= N
    out["weno"] = weno
    out["cfl"] = Cw * cfl_flops_per_wcell(system, ndim, V, N)
    per_it = (newton_flops_per_iteration if stiff else predictor_flops_per_iteration)(
        system, ndim, V, N)
    out["predictor"] = Cw * pred_iters_per_cell * per_it
    out["faces"] = face_points(nX, N) * face_point_flops(system, ndim, V, N)
    return out


def bytes_per_cell_update(nX, V, N):
    """Unfused algorithmic HBM bytes per cell-update, per stage (FP64)."""
    ndim = len(nX)
    C = Cb = Cw = 1
    for n in nX:
        C *= n
        Cb *= n + 2 * N
        Cw *= n + 2
    Nd = N ** ndim
    return {
        "ghost": 8 * V * (1 + Cb / C),
        "weno": 8 * V * (Cb / C) + 8 * V * Nd * Cw / C,
        "cfl": 8 * V * Nd * Cw / C,
        "predictor": 8 * V * Nd * (1 + N) * Cw / C,
        "fv": 8 * V * N * Nd * Cw / C + 16 * V,
    }


def faces_bytes_per_launch(nX, V, N):
    """Algorithmic HBM bytes of one k_faces launch: the predictor qh read
    once (N time nodes x N^d spatial nodes x V per w-cell) and the two
    contributions of every face point written (2 V each)."""
    Cw = 1
    for n in nX:
        Cw *= n + 2
    return 8.0 * (Cw * N * N ** len(nX) * V + face_points(nX, N) * 2 * V)
