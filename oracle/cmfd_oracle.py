"""CPU restatement of the reference's CMFD acceleration (numpy, FP64).

TEST INFRASTRUCTURE ONLY: the checker for the CMFD path of the CUDA
library.  Nothing in the product package imports this module.

Each step follows the reference, per FSR as the reference loops:
  * Cmfd::collapseXS (src/Cmfd.cpp:720-1000): flux-volume weighted total,
    nu-fission and scattering cross sections per coarse cell and coarse
    group, chi weighted by neutron production, D = sum_h rxn_h / (3
    sigma_t,h) / rxn, cell flux = rxn / volume (ZERO_SIGMA_T fallback for
    a zero reaction tally);
  * Cmfd::getSurfaceDiffusionCoefficient (src/Cmfd.cpp:1048-1170) with
    Cmfd::computeLarsensEDCFactor (src/Cmfd.cpp:1625-1650): vacuum
    2D/delta/(1+4D/delta), interface 2 D D' / (delta' D + delta D'), the
    correction term from the tallied net current, flux limiting after the
    first iteration, relaxation against the previous correction, no
    correction at the first iteration;
  * Cmfd::constructMatrices (src/Cmfd.cpp:1353-1500), entries below
    FLT_EPSILON dropped as there;
  * eigenvalueSolve / linearSolve / ddLinearSolve (src/linalg.cpp:25-176,
    179-385, 717-900): power iteration over red-black SOR with
    computeRMSE's integrated residual, at least 25 iterations of each, stop
    ratios 0.03 and 0.1, the diagonally dominated solve after a failure;
  * Cmfd::rescaleFlux and Cmfd::updateMOCFlux (src/Cmfd.cpp:1304-1350,
    1509-1560): ratios of new to old coarse flux, bounded to [0.05, 20]
    after the unbounded iterations;
  * Solver::computeEigenvalue with CMFD (src/Solver.cpp:1591-1680):
    sources, sweep with current tallies, addSourceToScalarFlux, CMFD keff
    and prolongation, normalizeFluxes, residual, source threshold
    0.01 * residual, storeFSRFluxes.
"""
from __future__ import annotations

import numpy as np

FLT_EPSILON = float(np.finfo(np.float32).eps)
ZERO_SIGMA_T = 1e-6
FLUX_EPSILON = 1e-25


class CmfdOracle:
    def __init__(self, problem, nx, ny, widths_x, widths_y, fsr_cell, end_face,
                 bc, group_of=None, edc_mu=None, edc_w=None, relaxation=0.7,
                 sor=1.5, flux_limiting=True, unbounded=0, linalg_tol=1e-7,
                 k_nearest=0, centroid=None, origin=(0.0, 0.0)):
        p = problem
        self.p = p
        self.nx, self.ny = int(nx), int(ny)
        self.C = self.nx * self.ny
        self.G = G = p.num_groups
        self.wx = np.asarray(widths_x, np.float64)
        self.wy = np.asarray(widths_y, np.float64)
        self.cell = np.ascontiguousarray(fsr_cell, np.int32)
        self.end_face = np.ascontiguousarray(end_face, np.int8)
        self.bc = [int(b) for b in bc]
        self.group_of = (np.arange(G) if group_of is None
                         else np.asarray(group_of, np.int64))
        self.E = E = int(self.group_of.max()) + 1
        self.edc_mu = np.zeros(0) if edc_mu is None else np.asarray(edc_mu, np.float64)
        self.edc_w = np.zeros(0) if edc_w is None else np.asarray(edc_w, np.float64)
        self.relaxation, self.sor = float(relaxation), float(sor)
        self.flux_limiting, self.unbounded = bool(flux_limiting), int(unbounded)
        self.tol_min = float(linalg_tol)
        M = p.num_materials
        self.st = p.sigma_t.reshape(M, G).astype(np.float64)
        self.nf = p.nu_sigma_f.reshape(M, G).astype(np.float64)
        self.chi = p.chi.reshape(M, G).astype(np.float64)
        self.ss = p.sigma_s.reshape(M, G, G).astype(np.float64)   # [m][dest][orig]
        self.vol = p.fsr_vol.astype(np.float64)
        self.mat = p.fsr_mat
        # neighbours [C][4] (faces x-min, y-min, x-max, y-max), -1 outside
        c = np.arange(self.C)
        ix, iy = c % self.nx, c // self.nx
        self.nbr = np.stack([np.where(ix > 0, c - 1, -1),
                             np.where(iy > 0, c - self.nx, -1),
                             np.where(ix < self.nx - 1, c + 1, -1),
                             np.where(iy < self.ny - 1, c + self.nx, -1)], 1)
        self.colors = [c[(ix + iy) % 2 == k] for k in (0, 1)]
        self.stencil = None
        if k_nearest > 0:
            self.stencil = knearest_stencils(self, int(k_nearest),
                                              np.asarray(centroid, np.float64).reshape(-1, 2),
                                              origin)
        self.reset()

    def reset(self, threshold=1e-5):
        self.keff = 1.0
        self.source_threshold = 0.1 * threshold
        self.dcorr_old = np.zeros((self.C, 4, self.E))
        self.dcorr_valid = False

    # ---------------------------------------------------------------- steps
    def _larsen(self, d, delta):
        if self.edc_mu.size == 0:
            return np.ones_like(d)
        mu = self.edc_mu[None, :]
        dd = d[..., None] if np.ndim(d) else d
        e = np.exp(-np.asarray(delta)[..., None] / (3.0 * dd * mu))
        alpha = (1.0 + e) / (1.0 - e) - 2.0 * (3.0 * dd * mu) / np.asarray(delta)[..., None]
        rho = (2.0 * mu * self.edc_w[None, :] * alpha).sum(-1)
        return 1.0 + delta * rho / (2.0 * d)

    def _collapse(self, phi):
        G, E, C = self.G, self.E, self.C
        m, cell = self.mat, self.cell
        phiv = phi * self.vol[:, None]                             # [R][G]
        rxn_h = np.zeros((C, G))
        trans_h = np.zeros((C, G))
        nuf_h = np.zeros((C, G))
        np.add.at(rxn_h, cell, phiv)
        np.add.at(trans_h, cell, self.st[m] * phiv)
        np.add.at(nuf_h, cell, self.nf[m] * phiv)
        # scattering out of group h into coarse group e'
        s_fsr = np.einsum("rgh,rh->rhg", self.ss[m], phiv)         # [R][h][g]
        s_coarse = np.zeros((s_fsr.shape[0], G, E))
        for g in range(G):
            s_coarse[:, :, self.group_of[g]] += s_fsr[:, :, g]
        scat_h = np.zeros((C, G, E))
        np.add.at(scat_h, cell, s_coarse)
        prod = (self.nf[m] * phiv).sum(1)                          # [R]
        chi_e = np.zeros((phi.shape[0], E))
        for h in range(G):
            chi_e[:, self.group_of[h]] += self.chi[m, h]
        chi_tally = np.zeros((C, E))
        np.add.at(chi_tally, cell, chi_e * prod[:, None])
        prod_c = np.zeros(C)
        np.add.at(prod_c, cell, prod)
        cell_vol = np.zeros(C)
        np.add.at(cell_vol, cell, self.vol)
        chi_c = np.where(np.abs(prod_c)[:, None] > 0,
                         chi_tally / np.where(prod_c == 0, 1, prod_c)[:, None], 0.0)
        sig_t = np.zeros((C, E))
        nu_f = np.zeros((C, E))
        dif = np.zeros((C, E))
        sig_s = np.zeros((C, E, E))
        phi_c = np.zeros((C, E))
        for e in range(E):
            hs = np.nonzero(self.group_of == e)[0]
            rxn = rxn_h[:, hs].sum(1)
            total = trans_h[:, hs].sum(1)
            nuf = nuf_h[:, hs].sum(1)
            scat = scat_h[:, hs, :].sum(1)
            ok = np.abs(trans_h[:, hs]) > np.abs(rxn_h[:, hs]) * FLT_EPSILON
            with np.errstate(divide="ignore", invalid="ignore"):
                dterm = np.where(ok, rxn_h[:, hs] / (3.0 * (trans_h[:, hs] / rxn_h[:, hs])), 0.0)
            dsum = dterm.sum(1)
            bad = rxn <= 0
            rxn = np.where(bad, ZERO_SIGMA_T, rxn)
            dsum = np.where(bad, ZERO_SIGMA_T, dsum)
            total = np.where(bad, ZERO_SIGMA_T, total)
            nuf = np.where(bad & (nuf != 0), ZERO_SIGMA_T, nuf)
            scat = np.where(bad[:, None], 0.0, scat)
            sig_t[:, e] = total / rxn
            nu_f[:, e] = nuf / rxn
            sig_s[:, e, :] = scat / rxn[:, None]
            dif[:, e] = dsum / rxn
            phi_c[:, e] = rxn / cell_vol
        return sig_t, nu_f, chi_c, dif, sig_s, phi_c, cell_vol

    def _build(self, it, cur, sig_t, nu_f, chi_c, dif, sig_s, phi_c, vol):
        C, E = self.C, self.E
        J = np.zeros((C, 4, E))
        for h in range(self.G):
            J[:, :, self.group_of[h]] += cur[:, :, h]
        ix, iy = np.arange(C) % self.nx, np.arange(C) // self.nx
        A = np.zeros((C, E, E))
        nb = np.zeros((C, 4, E))
        V = vol[:, None]
        idx = np.arange(E)
        A[:, idx, idx] += sig_t * V
        # A[c][e][g] -= sigma_s(g -> e) V
        ins = -np.transpose(sig_s, (0, 2, 1)) * V[:, :, None]
        A += np.where(np.abs(ins) > FLT_EPSILON, ins, 0.0)
        for f in range(4):
            xf = f in (0, 2)
            width = (self.wy[iy] if xf else self.wx[ix])[:, None]
            delta = (self.wx[ix] if xf else self.wy[iy])[:, None] * np.ones((1, E))
            n = self.nbr[:, f]
            d = dif * self._larsen(dif, delta)
            flux = phi_c
            dh = np.zeros((C, E))
            dt = np.zeros((C, E))
            inside = n >= 0
            if (~inside).any() and self.bc[f] == 0:
                o = ~inside
                cur_out = J[o, f, :] / width[o]
                dh[o] = 2.0 * d[o] / delta[o] / (1.0 + 4.0 * d[o] / delta[o])
                dt[o] = (dh[o] * flux[o] - cur_out) / flux[o]
            if inside.any():
                k = inside
                nn = n[k]
                nix, niy = nn % self.nx, nn // self.nx
                delta_n = (self.wx[nix] if xf else self.wy[niy])[:, None] * np.ones((1, E))
                dn = dif[nn] * self._larsen(dif[nn], delta_n)
                fn = phi_c[nn]
                j_in = J[nn, f ^ 2, :]
                h = 2.0 * d[k] * dn / (delta_n * d[k] + delta[k] * dn)
                current = (J[k, f, :] - j_in) / width[k]
                t = -(h * (fn - flux[k]) + current) / (fn + flux[k])
                if self.flux_limiting and it > 0:
                    lim = np.abs(t / h) > 1.0
                    h2 = np.where(current > 0, np.abs(current / (2.0 * flux[k])),
                                  np.abs(current / (2.0 * fn)))
                    t2 = -(h2 * (fn - flux[k]) + current) / (fn + flux[k])
                    h2 = np.maximum(h2, np.abs(t2))
                    h = np.where(lim, h2, h)
                    t = np.where(lim, t2, t)
                dh[k] = h
                dt[k] = t
            if self.dcorr_valid:
                dt = self.relaxation * dt + (1.0 - self.relaxation) * self.dcorr_old[:, f, :]
            if it == 0:
                dt = np.zeros_like(dt)
            self.dcorr_old[:, f, :] = dt
            A[:, idx, idx] += (dh - dt) * width
            nb[:, f, :] = np.where(inside[:, None], -(dh + dt) * width, 0.0)
        Mm = chi_c[:, :, None] * nu_f[:, None, :] * V[:, :, None]
        Mm = np.where(np.abs(Mm) > FLT_EPSILON, Mm, 0.0)
        self.dcorr_valid = True
        return A, nb, Mm

    @staticmethod
    def _rmse(x, y):
        a, b = x.sum(1), y.sum(1)
        ok = np.abs(b) > FLUX_EPSILON
        r = np.where(ok, ((a - b) / np.where(ok, b, 1.0)) ** 2, 0.0)
        return float(np.sqrt(r.sum() / max(x.shape[0], 1)))

    def _linear_solve(self, A, nb, Mm, x, b, tol):
        w = self.sor
        tol = max(self.tol_min, tol)
        E = self.E
        diag = A[:, np.arange(E), np.arange(E)]
        old_src = np.einsum("ceg,cg->ce", Mm, x)
        residual = initial = 0.0
        min_res = 1e6
        it = 0
        while it < 10000:
            for cells in self.colors:
                nbr = self.nbr[cells]
                for e in range(E):
                    d = diag[cells, e]
                    v = (1.0 - w) * x[cells, e] * (d / w)
                    row = A[cells, e, :].copy()
                    row[:, e] = 0.0
                    v -= (row * x[cells]).sum(1)
                    for f in range(4):
                        nf = nbr[:, f]
                        v -= np.where(nf >= 0, nb[cells, f, e] * x[np.maximum(nf, 0), e], 0.0)
                    v += b[cells, e]
                    x[cells, e] = v * (w / d)
            new_src = np.einsum("ceg,cg->ce", Mm, x)
            if it == 0:
                residual = initial = self._rmse(new_src, old_src)
            it += 1
            if it > 25:
                residual = self._rmse(new_src, old_src)
                min_res = min(min_res, residual)
                if (residual > 1e3 * min_res and min_res > 1e-10) or not np.isfinite(residual):
                    return False, it
                # IEEE division as in the reference: x / 0 never passes
                ratio = residual / initial if initial > 0 else float("inf")
                if ratio < 0.1 or residual < tol:
                    break
            if 24 < it < 10000:
                old_src = new_src
        return it < 10000, it

    def _dd_linear_solve(self, A, nb, Mm, x, b, tol):
        """ddLinearSolve (src/linalg.cpp:717-900)."""
        E = self.E
        idx = np.arange(E)
        off = np.abs(A).sum(2) - np.abs(A[:, idx, idx]) + np.abs(nb).sum(1)
        diag = A[:, idx, idx]
        dd = np.where(off > diag, off - diag, 0.0)
        A = A.copy()
        A[:, idx, idx] += dd
        new_src = np.einsum("ceg,cg->ce", Mm, x)
        initial, min_res = 0.0, 1e6
        for it in range(10000):
            old_src = new_src
            self._linear_solve(A, nb, Mm, x, b + dd * x, tol)
            new_src = np.einsum("ceg,cg->ce", Mm, x)
            res = self._rmse(new_src, old_src)
            if it == 0:
                initial = res if res >= 1e-14 else 1e-10
            min_res = min(min_res, res)
            if (res > 1e3 * min_res and min_res > 1e-10) or not np.isfinite(res):
                return False
            if res / initial < 0.1 or res < tol:
                break
        return True

    def _eigen_solve(self, A, nb, Mm, x, k, tol):
        tol = max(self.tol_min, tol)
        rows = x.size
        old_src = np.einsum("ceg,cg->ce", Mm, x)
        s = old_src.sum()
        old_src *= rows / s
        x *= rows * k / s
        initial = 0.0
        dd_mode = False
        for it in range(25000):
            ok = False
            if not dd_mode:
                ok, _ = self._linear_solve(A, nb, Mm, x, old_src, tol * 1e-1)
            if not ok:
                dd_mode = True
                ok = self._dd_linear_solve(A, nb, Mm, x, old_src, tol * 1e-1)
            if not ok:
                return -1.0, it + 1
            new_src = np.einsum("ceg,cg->ce", Mm, x)
            k = new_src.sum() / rows
            new_src /= k
            residual = self._rmse(new_src, old_src)
            if it == 0:
                initial = residual if residual >= 1e-14 else 1e-10
            old_src = new_src
            if (residual / initial < 0.03 or residual < self.tol_min) and it > 25:
                break
        return k, it + 1

    def compute_keff(self, it, phi, cur):
        """One Cmfd::computeKeff: returns (keff, ratio [cells][E])."""
        sig_t, nu_f, chi_c, dif, sig_s, phi_c, vol = self._collapse(phi)
        A, nb, Mm = self._build(it, cur, sig_t, nu_f, chi_c, dif, sig_s, phi_c, vol)
        x = phi_c.copy()
        k, self.power_iterations = self._eigen_solve(A, nb, Mm, x, self.keff,
                                                     self.source_threshold)
        if not (abs(k + 1.0) > FLT_EPSILON) or not np.isfinite(k):
            return self.keff, np.ones((self.C, self.E))
        self.keff = k
        new = x / np.einsum("ceg,cg->ce", Mm, x).sum()
        old = phi_c / np.einsum("ceg,cg->ce", Mm, phi_c).sum()
        ratio = np.where(np.abs(old) > FLUX_EPSILON, new / np.where(old == 0, 1, old), 0.0)
        self.old_flux, self.new_flux = old, new
        return k, ratio

    def update_ratios(self, it, ratio):
        """Cmfd::updateMOCFlux's ratio per FSR and coarse group: the cell's,
        or Cmfd::getUpdateRatio's k-nearest weighting; bounded to [0.05, 20]
        after the unbounded iterations."""
        if self.stencil is None:
            q = ratio[self.cell]
        else:
            q = np.stack([sum(c * ratio[cell] for cell, c in st)
                          for st in self.stencil])
        if it > self.unbounded:
            q = np.clip(q, 0.05, 20.0)
        return q


def knearest_stencils(cm, k, centroid, origin):
    """Cmfd::generateKNearestStencils (src/Cmfd.cpp:2887-2960) and the
    combination of Cmfd::getUpdateRatio (src/Cmfd.cpp:3178-3220), per FSR a
    list of (coarse cell, coefficient)."""
    cx = np.cumsum(cm.wx) - cm.wx / 2
    cy = np.cumsum(cm.wy) - cm.wy / 2
    out = []
    for r in range(centroid.shape[0]):
        c = int(cm.cell[r])
        ix, iy = c % cm.nx, c // cm.nx
        dx, dy = centroid[r, 0] - origin[0], centroid[r, 1] - origin[1]
        st = []
        for j in range(9):
            sx, sy = ix + j % 3 - 1, iy + j // 3 - 1
            if 0 <= sx < cm.nx and 0 <= sy < cm.ny:
                d = ((dx - cx[sx]) ** 2 + (dy - cy[sy]) ** 2) ** 0.5
            else:
                d = np.finfo(np.float64).max
            st.append((j, d))
        st = sorted(st, key=lambda e: e[1])          # stable, as libstdc++'s
        st = [e for e in st if e[1] <= 1e300][:k]    # insertion sort on 9
        total = 1e-10 + sum(d for _, d in st)
        st = [(j, 1.0 - d / total) for j, d in st]
        n = len(st)
        div = 1.0 if n == 1 else n - 1.0
        terms = [((iy + j // 3 - 1) * cm.nx + ix + j % 3 - 1, w / div)
                 for j, w in st if j != 4]
        terms.append((c, 1.0 if n == 1 else st[0][1] / div))
        out.append(terms)
    return out


def cmfd_eigenvalue(oracle, cm: CmfdOracle, max_iters=1000, res_type=1, tol=1e-5):
    """Solver::computeEigenvalue with CMFD on the transport oracle; returns
    the number of iterations (keff and fluxes are left in the oracle)."""
    p = oracle.p
    R, G = p.num_fsrs, p.num_groups
    oracle.keff = 1.0
    oracle.zero_track_fluxes()
    oracle.flatten(1.0)
    oracle.normalize()
    oracle.store()
    cm.reset(tol)
    k_prev = 1.0
    cur = np.zeros((cm.C, 4, G))
    its = 0
    stab = getattr(oracle, "stab_flux", None) is not None
    if stab:
        oracle.stab_flux[:] = 0.0
    for i in range(max_iters):
        if i > 0 and stab:      # Solver::computeEigenvalue, src/Solver.cpp:1616-1619
            oracle.compute_stabilizing_flux()
        oracle.compute_sources(i)
        cur[:] = 0.0
        oracle.sweep_currents(cm.cell, cm.end_face, cm.nx, cur)
        oracle.add_source()
        phi = oracle.phi.reshape(R, G).astype(np.float64)
        k, ratio = cm.compute_keff(i, phi, cur)
        oracle.keff = k
        scaled = phi * cm.update_ratios(i, ratio)[:, cm.group_of]
        oracle.phi[:] = scaled.ravel().astype(oracle.phi.dtype)
        if i > 0 and stab:      # after the CMFD update, src/Solver.cpp:1632-1635
            oracle.stabilize_flux()
        oracle.normalize()
        residual = oracle.residual_of(res_type)
        dk = int(1e5 * (k - k_prev))
        k_prev = k
        cm.source_threshold = 0.01 * (residual if residual > 0 else 1e-6)
        oracle.store()
        its += 1
        if residual < tol and abs(dk) < 1:
            break
    oracle.num_iterations = its
    oracle.residual = residual
    return its
