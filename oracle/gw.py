"""FP64 oracle of the GW/SCBA self-energy loop -- TEST INFRASTRUCTURE ONLY.

Restates the steps of gw_ephoton_3d_ijs (src/gw_mod.f90:78-1070) that make up
the GW self-energy loop (RGF, polarisation, screened interaction, self-energy,
mixing); the functions below are for one k-point, and ``*_k`` further down sum
over the k-pairs of nk = nky * nkz k-points and restrict P and Sigma to the
``ndiag`` band:

* energy correlation / convolution (src/fft_mod.f90:58-168, corr1d2 / conv1d2)
  on a uniform energy grid E_e = E_0 + e dE (e = 0..n-1) and the centred
  frequency grid w_m = (m - n/2) dE (m = 0..n-1):
      corr(X, Y)[m] = sum_e X[e] Y[e - (m - n/2)]
      conv(X, W)[e] = sum_m X[e - (m - n/2)] W[m]
  (terms whose index leaves [0, n) are dropped).  The reference's own
  'index'/'simple'/'fft' variants disagree with each other by one grid step
  (corr1d2 'fft' takes Z_(n - n/2 : n + n/2 - 1) while 'index' fills
  Z(i + n/2)); this is the mathematically centred form.
* polarisation (src/gw_mod.f90:444-519): Re G^{R,<,>} zeroed first (:444-446,
  the zeroed buffers are also the ones the self-energy convolutions read),
      P^<_ij = corr(G^<_ij, G^>_ji),  P^>_ij = corr(G^>_ij, G^<_ji),
      P^R_ij = corr(G^<_ij, conj G^R_ij) + corr(G^R_ij, G^<_ji),
  times -i dE / (2 pi) * spindeg / nk (:516-519), per slab-diagonal block.
* screened interaction: the reference's routine (green_rgf_calc_w, called at
  :597) is not in the repository, so W is restated per slab-diagonal block
      W^R = (I - V P^R)^-1 V,   W^{<,>} = W^R P^{<,>} W^R^+.
* self-energy (src/gw_mod.f90:646-698):
      S^< = conv(G^<, W^<), S^> = conv(G^>, W^>),
      S^R = conv(G^<, W^R) + conv(G^R, W^<) + conv(G^R, W^R),
  times i dE / (2 pi) / nk; S^R <- Re S^R + i Im(S^> - S^<)/2; symmetrised
  S <- (S + S^T)/2 (:731-743); linear mixing S <- S + alpha (S_new - S)
  (:747-749); edge blocks 1,2 <- 3 and nx-1,nx <- nx-2 (:950-959), applied
  here to the new iterate before mixing so that the fixed point is consistent.
* residual (no counterpart: the reference runs a fixed niter) =
  ||S_new - S||_F / ||S_new||_F over S^< and S^>.

Array layout: G and Sigma blocks as (nE, nx, nm, nm) numpy complex128.
Parity is unpinned against the reference (no GW fixture exists and the
reference's GW module does not build); this oracle pins the GPU path.
"""
from __future__ import annotations

import numpy as np

from . import rgf as orc


def corr(X, Y):
    """corr(X, Y)[..., m] = sum_e X[..., e] Y[..., e - (m - n/2)] along the last axis (FFT)."""
    n = X.shape[-1]
    L = 1 << int(np.ceil(np.log2(2 * n)))
    Z = np.fft.ifft(np.fft.fft(X, L) * np.fft.fft(Y[..., ::-1], L))
    t = np.arange(n) - n // 2 + n - 1
    return Z[..., t]


def conv(X, W):
    """conv(X, W)[..., e] = sum_m X[..., e - (m - n/2)] W[..., m] along the last axis (FFT)."""
    n = X.shape[-1]
    L = 1 << int(np.ceil(np.log2(2 * n)))
    Z = np.fft.ifft(np.fft.fft(X, L) * np.fft.fft(W, L))
    return Z[..., np.arange(n) + n // 2]


def corr_direct(X, Y):
    n = X.shape[-1]
    Z = np.zeros(X.shape[:-1] + (n,), dtype=np.complex128)
    for m in range(n):
        lag = m - n // 2
        for e in range(n):
            if 0 <= e - lag < n:
                Z[..., m] += X[..., e] * Y[..., e - lag]
    return Z


def conv_direct(X, W):
    n = X.shape[-1]
    Z = np.zeros(X.shape[:-1] + (n,), dtype=np.complex128)
    for e in range(n):
        for m in range(n):
            k = e - (m - n // 2)
            if 0 <= k < n:
                Z[..., e] += X[..., k] * W[..., m]
    return Z


def zero_real(*G):
    """Re G zeroed in place of the G buffers (src/gw_mod.f90:444-446); the same
    buffers feed both the polarisation and the self-energy convolutions."""
    return tuple(1j * A.imag for A in G)


def polarization(GR, GL, GG, dE, spindeg=2.0, nk=1):
    """P^{<,>,R} (nE, nx, nm, nm) from (Re-zeroed) G (nE, nx, nm, nm)."""
    gr, gl, gg = GR, GL, GG
    # series along energy: move E last
    s = lambda A: np.moveaxis(A, 0, -1)            # (nx, nm, nm, nE)
    t = lambda A: np.swapaxes(s(A), 1, 2)          # transposed partner G_ji
    PL = corr(s(gl), t(gg))
    PG = corr(s(gg), t(gl))
    PR = corr(s(gl), np.conj(s(gr))) + corr(s(gr), t(gl))
    fac = -1j * dE / (2 * np.pi) * spindeg / nk
    back = lambda A: np.moveaxis(A, -1, 0) * fac
    return back(PR), back(PL), back(PG)


def screened(V, PR, PL, PG):
    """W^R = (I - V P^R)^-1 V,  W^{<,>} = W^R P^{<,>} W^R^+ per (w, slab) block."""
    nm = V.shape[-1]
    I = np.eye(nm)
    WR = np.linalg.solve(I - V @ PR, np.broadcast_to(V, PR.shape))
    WRd = np.conj(np.swapaxes(WR, -1, -2))
    return WR, WR @ PL @ WRd, WR @ PG @ WRd


def self_energy(GR, GL, GG, WR, WL, WG, dE, nk=1):
    s = lambda A: np.moveaxis(A, 0, -1)
    SL = conv(s(GL), s(WL))
    SG = conv(s(GG), s(WG))
    SR = conv(s(GL), s(WR)) + conv(s(GR), s(WL)) + conv(s(GR), s(WR))
    fac = 1j * dE / (2 * np.pi) / nk
    back = lambda A: np.moveaxis(A, -1, 0) * fac
    SL, SG, SR = back(SL), back(SG), back(SR)
    SR = SR.real + 1j * (SG - SL).imag / 2
    sym = lambda A: (A + np.swapaxes(A, -1, -2)) / 2
    return sym(SR), sym(SL), sym(SG)


def copy_edges(S):
    nx = S.shape[1]
    if nx >= 5:
        S[:, 0] = S[:, 2]
        S[:, 1] = S[:, 2]
        S[:, nx - 1] = S[:, nx - 3]
        S[:, nx - 2] = S[:, nx - 3]
    return S


def green(E, H00, H10, nx, SR, SL, *, mu, temp, eta_lead=1e-3, sancho_nmax=100,
          sancho_reset=False):
    """G^{R,<,>} diagonal blocks (nE, nx, nm, nm) for self-energies SR, SL (green_RGF_RS).
    ``H00``: one on-site block (nm, nm) for every slab, or one per slab (nx, nm, nm).
    ``sancho_reset``: green_RGF_RS's lead decimation as written, restarting an unconverged
    run from H_SS = H_BB = H00 (src/gw_mod.f90:1440-1445)."""
    nE = len(E)
    nm = H00.shape[-1]
    Hii = list(H00) if H00.ndim == 3 else [H00] * nx
    GR = np.zeros((nE, nx, nm, nm), dtype=np.complex128)
    GL = np.zeros_like(GR)
    GG = np.zeros_like(GR)
    for ie, e in enumerate(E):
        o = orc.rgf_constblocksize(e, Hii, [H10] * (nx + 1), None, list(SL[ie]),
                                   list(SR[ie]), mul=mu[0], mur=mu[1], templ=temp[0],
                                   tempr=temp[1], eta_lead=eta_lead, sancho_nmax=sancho_nmax,
                                   sancho_tol=1e-100, sancho_reset=sancho_reset)
        GR[ie] = np.stack(o["G_r"])
        GL[ie] = np.stack(o["G_lesser"])
        GG[ie] = np.stack(o["G_greater"])
    return GR, GL, GG


def scba(E, H00, H10, V, nx, *, mu, temp, alpha=0.3, tol=1e-8, max_iter=60, spindeg=2.0,
         eta_lead=1e-3, history=None):
    """Plain linear-mixing SCBA; returns (SR, SL, SG, residuals)."""
    nE = len(E)
    nm = H00.shape[0]
    dE = E[1] - E[0]
    z = np.zeros((nE, nx, nm, nm), dtype=np.complex128)
    SR, SL, SG = z.copy(), z.copy(), z.copy()
    res = []
    for _ in range(max_iter):
        GR, GL, GG = green(E, H00, H10, nx, SR, SL, mu=mu, temp=temp, eta_lead=eta_lead)
        GR, GL, GG = zero_real(GR, GL, GG)
        PR, PL, PG = polarization(GR, GL, GG, dE, spindeg)
        WR, WL, WG = screened(V, PR, PL, PG)
        nR, nL, nG = self_energy(GR, GL, GG, WR, WL, WG, dE)
        nR, nL, nG = copy_edges(nR), copy_edges(nL), copy_edges(nG)
        r = np.sqrt(np.sum(np.abs(nL - SL) ** 2) + np.sum(np.abs(nG - SG) ** 2)) / \
            max(np.sqrt(np.sum(np.abs(nL) ** 2) + np.sum(np.abs(nG) ** 2)), 1e-300)
        res.append(r)
        if history is not None:
            history.append((SL.copy(), SG.copy(), nL.copy(), nG.copy()))
        SR = SR + alpha * (nR - SR)
        SL = SL + alpha * (nL - SL)
        SG = SG + alpha * (nG - SG)
        if r <= tol:
            break
    return SR, SL, SG, res


# ---------------------------------------------------------------- several k-points, band
#
# With nk = nky * nkz transverse k-points (ik = ikz + iky nkz, 0-based; the reference's
# ik = ikz + (iky-1) nkz, 1-based) the polarisation of momentum transfer q sums over the
# k-pairs (k, kd(k, q)) and the self-energy at k over (kd(k, q), q)
# (src/gw_mod.f90:476-512, 653-690):
#     P_q   = sum_k  corr(G_k, G_kd)          (each of the P^{<,>,R} terms)
#     S_k   = sum_q  conv(G_kd, W_q)          (each of the Sigma terms)
# with the scales -i dE/(2 pi) spindeg/nk and i dE/(2 pi)/nk, W_q from the Coulomb block
# V_q (Vii(:,:,:,iq), :597-600), and G, P, W, Sigma stored k-slowest as the reference's
# (nm, nm, nx, nE, nk) arrays: numpy (nk, nE, nx, nm, nm).  ndiag keeps only the
# elements |i - j| <= ndiag of P and Sigma (:473-475, 527-555, 650-654, 705-730);
# None keeps the full blocks.


def kd_index(ik, iq, nky, nkz):
    """0-based k-pair partner ikd of ik and iq: per direction ikzd = ikz - iqz + nkz/2
    (1-based, integer division) wrapped once into [1, nkz], and 1 when nkz = 1
    (src/gw_mod.f90:478-487, 658-667)."""
    iky, ikz = divmod(ik, nkz)
    iqy, iqz = divmod(iq, nkz)
    kzd = (ikz - iqz + nkz // 2 - 1) % nkz
    kyd = (iky - iqy + nky // 2 - 1) % nky
    return kzd + kyd * nkz


def band_mask(nm, ndiag):
    """True where |i - j| <= ndiag (all True for ndiag None), the elements the reference's
    P and Sigma loops compute (src/gw_mod.f90:471-475) and its zeroing keeps (:527-555)."""
    i = np.arange(nm)
    if ndiag is None or ndiag < 0:
        return np.ones((nm, nm), dtype=bool)
    return np.abs(i[:, None] - i[None, :]) <= ndiag


def _pol_terms(grk, glk, ggk, grd, gld, ggd):
    """Unscaled (P^R, P^<, P^>) of one k-pair: G at k (grk, ...) and at kd (grd, ...),
    each (nE, nx, nm, nm)."""
    s = lambda A: np.moveaxis(A, 0, -1)
    t = lambda A: np.swapaxes(s(A), 1, 2)
    PL = corr(s(glk), t(ggd))
    PG = corr(s(ggk), t(gld))
    PR = corr(s(glk), np.conj(s(grd))) + corr(s(grk), t(gld))
    back = lambda A: np.moveaxis(A, -1, 0)
    return back(PR), back(PL), back(PG)


def _sigma_terms(grd, gld, ggd, wr, wl, wg):
    """Unscaled (S^R, S^<, S^>) of one pair: G at kd, W at q, each (nE, nx, nm, nm)."""
    s = lambda A: np.moveaxis(A, 0, -1)
    SL = conv(s(gld), s(wl))
    SG = conv(s(ggd), s(wg))
    SR = conv(s(gld), s(wr)) + conv(s(grd), s(wl)) + conv(s(grd), s(wr))
    back = lambda A: np.moveaxis(A, -1, 0)
    return back(SR), back(SL), back(SG)


def polarization_k(GR, GL, GG, dE, nky, nkz, spindeg=2.0, ndiag=None):
    """P^{R,<,>} (nk, nE, nx, nm, nm) of the k-pair sums from Re-zeroed G of the same
    shape, banded by ndiag."""
    nk = nky * nkz
    P = [np.zeros_like(GR) for _ in range(3)]
    for iq in range(nk):
        for ik in range(nk):
            kd = kd_index(ik, iq, nky, nkz)
            for acc, v in zip(P, _pol_terms(GR[ik], GL[ik], GG[ik], GR[kd], GL[kd], GG[kd])):
                acc[iq] += v
    m = band_mask(GR.shape[-1], ndiag)
    fac = -1j * dE / (2 * np.pi) * spindeg / nk
    return tuple(A * fac * m for A in P)


def screened_k(V, PR, PL, PG):
    """W per momentum transfer q with its own Coulomb block V[q] (nk, nm, nm)."""
    out = [screened(V[q], PR[q], PL[q], PG[q]) for q in range(PR.shape[0])]
    return tuple(np.stack([o[c] for o in out]) for c in range(3))


def self_energy_k(GR, GL, GG, WR, WL, WG, dE, nky, nkz, ndiag=None):
    """Sigma^{R,<,>} (nk, nE, nx, nm, nm) of the k-pair sums, recombined
    (Re S^R + i Im(S^> - S^<)/2), banded by ndiag and symmetrised."""
    nk = nky * nkz
    S = [np.zeros_like(GR) for _ in range(3)]
    for ik in range(nk):
        for iq in range(nk):
            kd = kd_index(ik, iq, nky, nkz)
            for acc, v in zip(S, _sigma_terms(GR[kd], GL[kd], GG[kd], WR[iq], WL[iq], WG[iq])):
                acc[ik] += v
    m = band_mask(GR.shape[-1], ndiag)
    fac = 1j * dE / (2 * np.pi) / nk
    SR, SL, SG = (A * fac * m for A in S)
    SR = SR.real + 1j * (SG - SL).imag / 2
    sym = lambda A: (A + np.swapaxes(A, -1, -2)) / 2
    return sym(SR), sym(SL), sym(SG)


def gw_map_k(E, H00k, H10k, V, nx, SR, SL, *, nky, nkz, mu, temp, spindeg=2.0,
             eta_lead=1e-3, ndiag=None, sancho_reset=False):
    """One evaluation of the SCBA map at nk = nky * nkz k-points.  H00k (nk, [nx,] nm, nm),
    H10k (nk, nm, nm), V (nk, nm, nm); SR, SL (nk, nE, nx, nm, nm).  Returns the new
    (SR, SL, SG) with the edge blocks copied."""
    nk = nky * nkz
    dE = E[1] - E[0]
    G = [zero_real(*green(E, H00k[k], H10k[k], nx, SR[k], SL[k], mu=mu, temp=temp,
                          eta_lead=eta_lead, sancho_reset=sancho_reset)) for k in range(nk)]
    GR, GL, GG = (np.stack([g[c] for g in G]) for c in range(3))
    P = polarization_k(GR, GL, GG, dE, nky, nkz, spindeg, ndiag)
    W = screened_k(V, *P)
    N = self_energy_k(GR, GL, GG, *W, dE, nky, nkz, ndiag)
    # copy_edges works on axis 1 = slabs: apply per k
    return tuple(np.stack([copy_edges(A[k]) for k in range(nk)]) for A in N)


def scba_k(E, H00k, H10k, V, nx, *, nky, nkz, mu, temp, alpha=0.3, tol=1e-8, max_iter=60,
           spindeg=2.0, eta_lead=1e-3, ndiag=None):
    """Plain linear-mixing SCBA over k-points; returns (SR, SL, SG, residuals)."""
    nk, nm = nky * nkz, H00k.shape[-1]
    z = np.zeros((nk, len(E), nx, nm, nm), dtype=np.complex128)
    SR, SL, SG = z.copy(), z.copy(), z.copy()
    res = []
    for _ in range(max_iter):
        nR, nL, nG = gw_map_k(E, H00k, H10k, V, nx, SR, SL, nky=nky, nkz=nkz, mu=mu,
                              temp=temp, spindeg=spindeg, eta_lead=eta_lead, ndiag=ndiag)
        r = np.sqrt(np.sum(np.abs(nL - SL) ** 2) + np.sum(np.abs(nG - SG) ** 2)) / \
            max(np.sqrt(np.sum(np.abs(nL) ** 2) + np.sum(np.abs(nG) ** 2)), 1e-300)
        res.append(r)
        SR = SR + alpha * (nR - SR)
        SL = SL + alpha * (nL - SL)
        SG = SG + alpha * (nG - SG)
        if r <= tol:
            break
    return SR, SL, SG, res


def energies_to_ijs_2(bufs, nm, nx, nk, local_ne):
    """energies_to_ijs_2 (src/gw_mod.f90:41-73) on every rank at once, MPI_Alltoall done by
    hand.  ``bufs[r]``: rank r's flat buffer, g(1:nm, 1:nm, 1:nx, 1:local_ne, 1:nk) in
    Fortran order.  Returns rank r's buffer after the call as a numpy array indexed
    [e, s, k, x, a] (Fortran p3(1:local_ne, 1:comm_size, 1:nk, 1:nx, 1:local_nij)), i.e.
    global energy s*local_ne + e of element r*local_nij + a.  Needs nm*nm divisible by the
    rank count, as the reference's partition does."""
    size = len(bufs)
    local_nij = nm * nm // size
    count = local_nij * nx * local_ne * nk
    tmp0 = []
    for b in bufs:
        p0 = np.reshape(b[:count * size], (local_nij, size, nx, local_ne, nk), order="F")
        # p1 = reshape(p0, shape(p1), order=[1, 5, 2, 3, 4]): p1(a, x, e, k, r) = p0(a, r, x, e, k)
        tmp0.append(np.transpose(p0, (0, 2, 3, 4, 1)).reshape(-1, order="F"))
    # MPI_Alltoall: block s of rank r's receive buffer is block r of rank s's send buffer
    tmp1 = [np.concatenate([tmp0[s][r * count:(r + 1) * count] for s in range(size)])
            for r in range(size)]
    out = []
    for r in range(size):
        p2 = np.reshape(tmp1[r], (local_nij, nx, local_ne, nk, size), order="F")
        # p3 = reshape(p2, shape(p3), order=[5, 4, 1, 3, 2]): p3(e, s, k, x, a) = p2(a, x, e, k, s)
        out.append(np.transpose(p2, (2, 4, 3, 1, 0)))
    return out


def ijs_to_energies_2(outs, nm, nx, nk, local_ne):
    """The inverse of ``energies_to_ijs_2`` (ijs_to_energies_2 is called at
    src/gw_mod.f90:522-524, 700-702 but its source is absent): per-rank arrays [e, s, k, x, a]
    back to flat Fortran-order g(1:nm, 1:nm, 1:nx, 1:local_ne, 1:nk) buffers."""
    size = len(outs)
    local_nij = nm * nm // size
    count = local_nij * nx * local_ne * nk
    tmp1 = [np.transpose(o, (4, 3, 0, 2, 1)).reshape(-1, order="F") for o in outs]
    tmp0 = [np.concatenate([tmp1[s][r * count:(r + 1) * count] for s in range(size)])
            for r in range(size)]
    bufs = []
    for r in range(size):
        p1 = np.reshape(tmp0[r], (local_nij, nx, local_ne, nk, size), order="F")
        bufs.append(np.transpose(p1, (0, 4, 1, 2, 3)).reshape(-1, order="F"))
    return bufs


def coulomb_blocks(nm, spacing_nm=0.25, strength=14.4):
    """V_ij = 14.4 / (|r_i - r_j| + 1) eV on a 1-D grid of 0.25 nm (orbital index x spacing)."""
    r = np.arange(nm) * spacing_nm
    return strength / (np.abs(r[:, None] - r[None, :]) + 1.0)


# e-photon prefactor (hbar/m0)^2 / (2 eps0 c0^3), src/gw_mod.f90:92, constants of
# src/static.f90:10-14
PHOTON_PRE_FACT = ((1.0546e-34 / 9.109e-31) ** 2) / (2.0 * 8.854e-12 * 2.998e8 ** 3)


def ephoton_sigma(M, GL, GG, nop, pre_fact, intensity, hw, halo=False):
    """calc_sigma_ephoton_monochromatic_ext (src/gw_mod.f90:1075-1122), row-major numpy.

    M (nx, nm, nm); GL, GG (nE + 2 nop, nx, nm, nm) when ``halo`` (energy e at index
    e + nop) else (nE, nx, nm, nm) with zeros beyond the grid.  Returns (SR, SL, SG),
    each (nE, nx, nm, nm): Sigma^<> = M [G(e - nop) + G(e + nop)] M * pre_fact *
    intensity / hw^2 and Sigma^R = i Im(Sigma^> - Sigma^<) / 2."""
    def ext(G):
        if halo:
            return G
        Z = np.zeros((G.shape[0] + 2 * nop,) + G.shape[1:], dtype=np.complex128)
        Z[nop:nop + G.shape[0]] = G
        return Z

    nE = GL.shape[0] - (2 * nop if halo else 0)
    out = []
    for G in (GL, GG):
        Ge = ext(G)
        A = Ge[0:nE] + Ge[2 * nop:2 * nop + nE]  # ie2 -+ nop with ie2 = ie + nop
        S = np.einsum("xab,exbc,xcd->exad", M, A, M)
        out.append(S * pre_fact * intensity / hw ** 2)
    SL, SG = out
    return 1j * (SG - SL).imag / 2.0, SL, SG
