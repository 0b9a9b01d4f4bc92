"""FP64 CPU oracle for the recursive Green's function (RGF) sweep.

TEST INFRASTRUCTURE ONLY.  This module is the checker: the CUDA product path
never imports it.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may call it.

It restates, with numpy + scipy LAPACK (the same zgetrf/zgetrs sequence the
reference issues), the algorithm of

* ``sancho``                  src/cuda_rgf_mod.f90:657-765 (GPU variant, eta=1e-5, 50 iters)
                              src/rgf_mod.f90:482-568     (CPU variant, identical arithmetic)
                              src/gw_mod.f90:1378-1464    (GW variant, eta=1e-3, 100 iters,
                                                           reset H_SS=H_BB=H00 on nmax)
* ``rgf_constblocksize``      src/cuda_rgf_mod.f90:53-413  (the routine negf_solve calls,
                              src/negf_mod.f90:122-125)
* ``rgf_variableblock_forward`` src/rgf_mod.f90:46-269     (CPU variant; its contact-Fermi and
                              ``tr`` sign conventions differ, see ``quirks``)
* ``cell_traces``             src/output_mod.f90:37-59     (per-cell diagonal traces behind the
                              ldos/ndos/pdos files)

Index convention (0-based, mathematical, independent of memory layout):
``Hii[l]`` is the on-site block of slab l, ``H1i[l]`` is the coupling
H_{l,l-1} (rows in slab l, columns in slab l-1); ``H1i[0]`` couples the left
lead to slab 0 and ``H1i[nx]`` couples slab nx-1 to the right lead, exactly
the reference's ``H1i(1:nx+1)`` (src/deviceHam_mod.f90:278-286).

Parity is pinned: ``tests/test_oracle_golden.py`` reproduces the reference's
own outputs in test_cnt/ (sancho_g00.dat, sancho_gbb.dat, ldos/ndos/pdos0000.dat).
"""
from __future__ import annotations

import numpy as np
from scipy.linalg import lapack

BOLTZ = 8.61734e-05  # eV/K, src/cuda_rgf_mod.f90:22, src/rgf_mod.f90:38


def ferm(a):
    """Fermi function 1/(1+exp(a)) (src/cuda_rgf_mod.f90:859-863)."""
    return 1.0 / (1.0 + np.exp(a))


def invert(A):
    """LU inverse by zgetrf + zgetrs(I) as in src/cuda_rgf_mod.f90:624-654.

    Returns (Ainv, info).  Unlike the reference (which zeroes A or aborts),
    the status is returned to the caller.
    """
    n = A.shape[0]
    lu, piv, info1 = lapack.zgetrf(np.asarray(A, dtype=np.complex128))
    if info1 != 0:
        return np.zeros_like(A), int(info1)
    x, info2 = lapack.zgetrs(lu, piv, np.eye(n, dtype=np.complex128))
    return x, int(info2)


def dag(A):
    return A.conj().T


def sancho(E, S00, H00, H10, eta=1e-5, nmax=50, tol=1e-100, reset_on_nmax=False):
    """Lopez-Sancho decimation (src/cuda_rgf_mod.f90:657-765).

    Per iteration (src/cuda_rgf_mod.f90:687-715):
      A = (z S - H_BB)^-1;  B = A H_10;  C = H_01 B
      H_SS += C; H_BB += C
      C = H_10 B;  B = A H_01;  A = H_10 B
      H_10 = C;  H_BB += A;  C = H_01 B;  H_01 = C
      error = sum |C_kj|; exit if error < tol.
    ``reset_on_nmax`` is the GW variant's reset (src/gw_mod.f90:1440-1445).
    Returns (G00, GBB, iterations, error, info) with G00 the surface and GBB
    the bulk Green's function.
    """
    z = complex(E, eta)
    H_BB = np.array(H00, dtype=np.complex128)
    H_SS = H_BB.copy()
    H_10 = np.array(H10, dtype=np.complex128)
    H_01 = dag(H_10)
    info = 0
    it = 0
    error = np.inf
    for it in range(1, nmax + 1):
        A, inf = invert(z * S00 - H_BB)
        info = info or inf
        B = A @ H_10
        C = H_01 @ B
        H_SS = H_SS + C
        H_BB = H_BB + C
        C = H_10 @ B
        B = A @ H_01
        A = H_10 @ B
        H_10 = C
        H_BB = H_BB + A
        C = H_01 @ B
        H_01 = C
        error = float(np.sum(np.abs(C)))
        if abs(error) < tol:
            break
        if it == nmax and reset_on_nmax:
            H_SS = np.array(H00, dtype=np.complex128)
            H_BB = np.array(H00, dtype=np.complex128)
    G00, inf1 = invert(z * S00 - H_SS)
    GBB, inf2 = invert(z * S00 - H_BB)
    return G00, GBB, it, error, (info or inf1 or inf2)


# Reference quirks: the GPU routine as written (src/cuda_rgf_mod.f90).
QUIRKS_CUDA = dict(
    left_fermi=("l", "l"),  # Sigma^<_L uses (mul, TEMPl)            src/cuda_rgf_mod.f90:113
    right_fermi=("r", "l"),  # Sigma^<_R uses (mur, TEMPl)          src/cuda_rgf_mod.f90:242,256,264
    tre_fermi=("l", "r"),  # tre uses (mul, TEMPr)                  src/cuda_rgf_mod.f90:388,396
    tr_sign=-1.0,          # tr = -Re Tr[...]                       src/cuda_rgf_mod.f90:271-277
    sigr_times_s=False,    # interior adds Sigma_ph^R without *S    src/cuda_rgf_mod.f90:142
    greater_from_glp=True,  # G^> recursion propagates Glp == 0     src/cuda_rgf_mod.f90:78,351-372
    back_coupling="l",     # backward step at slab l uses H1i(l)    src/cuda_rgf_mod.f90:284
    jdens="cuda",          # cur = H10^+(...) - H10(...)            src/cuda_rgf_mod.f90:293-318
)
# What produced the reference's test_cnt/ outputs: the GPU routine's pairings,
# but G^> = G^< + (G - G^+) in every slab (the Glp==0 recursion is refuted by
# pdos0000.dat: 841 of 3000 rows differ in the printed digits).
QUIRKS_GOLDEN = dict(QUIRKS_CUDA, greater_from_glp=False)

QUIRKS_CPU = dict(
    left_fermi=("r", "r"),  # Sigma^<_L uses (mur, TEMPr)            src/rgf_mod.f90:100
    right_fermi=("l", "l"),  # Sigma^<_R uses (mul, TEMPl)          src/rgf_mod.f90:182,191,193
    tre_fermi=("r", "r"),  # tre uses (mur, TEMPr)                  src/rgf_mod.f90:258,260
    tr_sign=+1.0,          # tr = +Re Tr[...]                       src/rgf_mod.f90:196-202
    sigr_times_s=True,     #                                        src/rgf_mod.f90:120-121
    greater_from_glp=False,  # G^> = G^< + G - G^+ in every slab    src/rgf_mod.f90:249
    back_coupling="l",     # backward step at slab l uses H1i(l)    src/rgf_mod.f90:215-245
    jdens="cpu",           # Jdens = -2 H10^+ (...)                 src/rgf_mod.f90:215-221
    right_coupling="nx+1",  # right lead decimated with H1i(nx+1)   src/rgf_mod.f90:153
)
# Physically consistent conventions for blocks of different sizes: the backward step
# couples slab l to l+1 through H_{l+1,l} = H1i[l+1] (the reference's H1i(l) only fits
# when neighbouring blocks have equal size), each lead through its own coupling block.
QUIRKS_VARIABLE = dict(QUIRKS_CPU, back_coupling="next")


def _diags(blocks):
    """(nx, nm) diagonals for equal blocks; packed (sum n_l,) when sizes vary."""
    d = [np.diag(x) for x in blocks]
    return np.stack(d) if len({len(x) for x in d}) == 1 else np.concatenate(d)


def _coupling(H1i, l, mode):
    # The reference's backward loop couples slab l to l+1 through H1i(l)
    # (1-based), i.e. 0-based H1i[l]; the physically consistent block is
    # H1i[l+1].  They coincide whenever the coupling is slab-independent.
    return H1i[l] if mode == "l" else H1i[l + 1]


def rgf_constblocksize(E, Hii, H1i, Sii=None, sigma_lesser_ph=None, sigma_r_ph=None,
                       mul=0.0, mur=0.0, templ=300.0, tempr=300.0, *, quirks=None,
                       eta_lead=1e-5, sancho_nmax=50, sancho_tol=1e-100,
                       interior_eta=0.0, want_blocks=True, sancho_reset=False):
    """One (E,k) point of the ballistic/phonon RGF, src/cuda_rgf_mod.f90:53-413.

    ``sancho_reset``: the leads use green_RGF_RS's decimation, which restarts an
    unconverged run from H_SS = H_BB = H00 (src/gw_mod.f90:1440-1445).

    Returns a dict with G_r, G_lesser, G_greater, Jdens (lists of nx blocks,
    when ``want_blocks``), their diagonals, tr, tre, the Sancho surface/bulk
    Green's functions of both leads and a LAPACK info flag.
    """
    q = dict(QUIRKS_GOLDEN if quirks is None else quirks)
    nx = len(Hii)
    sizes = [h.shape[0] for h in Hii]  # block sizes may vary along the device
    if Sii is None:
        Sii = [np.eye(n, dtype=np.complex128) for n in sizes]
    zeros = [np.zeros((n, n), dtype=np.complex128) for n in sizes]
    if sigma_lesser_ph is None:
        sigma_lesser_ph = zeros
    if sigma_r_ph is None:
        sigma_r_ph = zeros
    z = complex(E, interior_eta)

    def fermi(which):
        mu = {"l": mul, "r": mur}[which[0]]
        T = {"l": templ, "r": tempr}[which[1]]
        return ferm((E - mu) / (BOLTZ * T))

    info = 0
    # ---- left contact (src/cuda_rgf_mod.f90:90-134)
    S00 = Sii[0]
    H00 = Hii[0] + sigma_r_ph[0] @ S00
    H10 = H1i[0]
    G00L, GBBL, itL, errL, inf = sancho(E, S00, H00, dag(H10), eta=eta_lead,
                                        nmax=sancho_nmax, tol=sancho_tol,
                                        reset_on_nmax=sancho_reset)
    info = info or inf
    sigmal = H10 @ G00L @ dag(H10)
    fl = fermi(q["left_fermi"][0] + q["left_fermi"][1])
    sig = -(sigmal - dag(sigmal)) * fl + sigma_lesser_ph[0] @ S00
    g, inf = invert(z * S00 - H00 - sigmal)
    info = info or inf
    Gl = [None] * nx
    Gln = [None] * nx
    Gl[0] = g
    Gln[0] = g @ sig @ dag(g)
    # ---- forward sweep (src/cuda_rgf_mod.f90:140-188)
    for l in range(1, nx - 1):
        sr = sigma_r_ph[l] @ Sii[l] if q["sigr_times_s"] else sigma_r_ph[l]
        H00 = Hii[l] + sr
        H10 = H1i[l]
        C = H10 @ Gl[l - 1] @ dag(H10)
        g, inf = invert(z * Sii[l] - H00 - C)
        info = info or inf
        C = H10 @ Gln[l - 1] @ dag(H10) + sigma_lesser_ph[l] @ Sii[l]
        Gl[l] = g
        Gln[l] = g @ C @ dag(g)
    # ---- right contact (src/cuda_rgf_mod.f90:192-277)
    S00 = Sii[nx - 1]
    H00 = Hii[nx - 1] + sigma_r_ph[nx - 1] @ S00
    # lead coupling: H1i(nx) in the GPU routine (src/cuda_rgf_mod.f90:157-159), the lead's
    # own H1i(nx+1) in the CPU routine (src/rgf_mod.f90:153); device coupling H1i(nx)
    Hlead = H1i[nx - 1] if q.get("right_coupling", "nx") == "nx" else H1i[nx]
    G00R, GBBR, itR, errR, inf = sancho(E, S00, H00, Hlead, eta=eta_lead,
                                        nmax=sancho_nmax, tol=sancho_tol,
                                        reset_on_nmax=sancho_reset)
    info = info or inf
    sigmar = dag(Hlead) @ G00R @ Hlead
    H10 = H1i[nx - 1]
    C = H10 @ Gl[nx - 2] @ dag(H10)
    GNN, inf = invert(z * S00 - H00 - sigmar - C)
    info = info or inf
    fr = fermi(q["right_fermi"][0] + q["right_fermi"][1])
    gam_r = -(sigmar - dag(sigmar))
    sig = gam_r * fr + H10 @ Gln[nx - 2] @ dag(H10) + sigma_lesser_ph[nx - 1] @ S00
    Gn = GNN @ sig @ dag(GNN)
    Gp = Gn + (GNN - dag(GNN))
    B = (gam_r * fr) @ Gp
    Cc = (gam_r * (fr - 1.0)) @ Gn
    tr = q["tr_sign"] * float(np.real(np.trace(B - Cc)))
    G_r = [None] * nx
    G_l = [None] * nx
    G_g = [None] * nx
    Jd = [None] * nx
    G_r[nx - 1] = GNN
    G_l[nx - 1] = Gn
    G_g[nx - 1] = Gp
    Jd[nx - 1] = (B - Cc) if q["jdens"] == "cpu" else zeros[nx - 1]
    # ---- backward sweep (src/cuda_rgf_mod.f90:283-381)
    G00 = GNN
    for l in range(nx - 2, -1, -1):
        H10 = _coupling(H1i, l, q["back_coupling"])
        g = Gl[l]
        gn = Gln[l]
        if q["jdens"] == "cuda":
            cur = dag(H10) @ (Gn @ H10 @ dag(g) + G00 @ H10 @ gn)
            cur = cur - H10 @ (g @ dag(H10) @ Gn + gn @ dag(H10) @ dag(G00))
        else:
            cur = -2.0 * (dag(H10) @ (Gn @ H10 @ dag(g) + G00 @ H10 @ gn))
        GN0 = g @ dag(H10) @ G00
        Gr_new = g + GN0 @ H10 @ g
        Gn_new = (gn + g @ dag(H10) @ Gn @ H10 @ dag(g)
                  + GN0 @ H10 @ gn + gn @ dag(H10) @ dag(GN0))
        if q["greater_from_glp"]:
            # Glp is allocated and zeroed but never filled (src/cuda_rgf_mod.f90:78)
            Gp_new = g @ dag(H10) @ Gp @ H10 @ dag(g)
        else:
            Gp_new = Gn_new + (Gr_new - dag(Gr_new))
        G00, Gn, Gp = Gr_new, Gn_new, Gp_new
        G_r[l], G_l[l], G_g[l], Jd[l] = G00, Gn, Gp, cur
    # ---- left-contact current (src/cuda_rgf_mod.f90:387-407)
    Gp_1 = Gn + (G00 - dag(G00))
    gam_l = -(sigmal - dag(sigmal))
    fe = fermi(q["tre_fermi"][0] + q["tre_fermi"][1])
    B = (gam_l * fe) @ Gp_1
    Cc = (gam_l * (fe - 1.0)) @ Gn
    tre = float(np.real(np.trace(B - Cc)))
    out = dict(tr=tr, tre=tre, info=info,
               sancho_left=(G00L, GBBL, itL, errL), sancho_right=(G00R, GBBR, itR, errR),
               diag_Gr=_diags(G_r), diag_Gl=_diags(G_l), diag_Gg=_diags(G_g))
    if want_blocks:
        out.update(G_r=G_r, G_lesser=G_l, G_greater=G_g, Jdens=Jd, Gl=Gl, Gln=Gln)
    return out


def rgf_variableblock_forward(E, Hii, H1i, Sii=None, sigma_lesser_ph=None, sigma_r_ph=None,
                              mul=0.0, mur=0.0, templ=300.0, tempr=300.0, **kw):
    """CPU-variant semantics (src/rgf_mod.f90:46-269): same sweep, CPU quirks."""
    return rgf_constblocksize(E, Hii, H1i, Sii, sigma_lesser_ph, sigma_r_ph, mul, mur,
                              templ, tempr, quirks=QUIRKS_CPU, **kw)


def caroli_transmission(E, Hii, H1i, Sii=None, *, eta_lead=1e-5, sancho_nmax=50,
                        sancho_tol=1e-100, interior_eta=0.0, sigma_r_ph=None):
    """Landauer/Caroli T(E) = Tr[Gamma_L G_{1N}^+ Gamma_R G_{N1}] ... in the
    form Tr[Gamma_R G_{N1} Gamma_L G_{N1}^+], from the left-connected chain
    P_0 = g_0, P_l = g_l H_{l,l-1} P_{l-1}, G_{N1} = G_NN H_{N,N-1} P_{N-2}.
    Leads and sweep follow ``rgf_constblocksize`` (same z, same Sancho).
    Not a reference routine: the reference only reports the terminal-current
    spectra ``tr``/``tre``; T(E) is the quantity the benchmark asks for.
    Also returns the per-slab LDOS traces -2 Im Tr G^R_ll (for cross-checks).
    """
    nx = len(Hii)
    nm = Hii[0].shape[0]
    I = np.eye(nm, dtype=np.complex128)
    if Sii is None:
        Sii = [I] * nx
    zero = np.zeros((nm, nm), dtype=np.complex128)
    if sigma_r_ph is None:
        sigma_r_ph = [zero] * nx
    z = complex(E, interior_eta)
    H00 = Hii[0] + sigma_r_ph[0] @ Sii[0]
    G00L = sancho(E, Sii[0], H00, dag(H1i[0]), eta=eta_lead, nmax=sancho_nmax, tol=sancho_tol)[0]
    sigl = H1i[0] @ G00L @ dag(H1i[0])
    g, _ = invert(z * Sii[0] - H00 - sigl)
    P = g
    for l in range(1, nx - 1):
        C = H1i[l] @ g @ dag(H1i[l])
        g, _ = invert(z * Sii[l] - Hii[l] - sigma_r_ph[l] - C)
        P = g @ H1i[l] @ P
    H00 = Hii[nx - 1] + sigma_r_ph[nx - 1] @ Sii[nx - 1]
    H10 = H1i[nx - 1]
    G00R = sancho(E, Sii[nx - 1], H00, H10, eta=eta_lead, nmax=sancho_nmax, tol=sancho_tol)[0]
    sigr = dag(H10) @ G00R @ H10
    GNN, _ = invert(z * Sii[nx - 1] - H00 - sigr - H10 @ g @ dag(H10))
    GN1 = GNN @ H10 @ P
    gam_l = 1j * (sigl - dag(sigl))
    gam_r = 1j * (sigr - dag(sigr))
    return float(np.real(np.trace(gam_r @ GN1 @ gam_l @ dag(GN1))))


def cell_traces(diag, NB, NS):
    """Per-cell diagonal traces (src/output_mod.f90:37-59) for one point.

    ``diag``: (nx, nm) diagonals of the slab blocks with nm = NB*NS.
    Returns (nx*NS,) complex traces, cell-major along transport.
    """
    nx = diag.shape[0]
    return diag.reshape(nx, NS, NB).sum(axis=2).reshape(nx * NS)
