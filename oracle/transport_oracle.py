"""CPU oracle of the grid tracer transport (test infrastructure only).

A numpy restatement of src/dynamics/aeros_transport.f90: positive-definite
finite-volume transport of a grid tracer q by the winds (u, v) and the air-mass
budget of the surface pressure, sub-stepped at the largest total Courant
number.  Used by tests/ to check the CUDA path; nothing in the product imports
it.  Arrays are (nlev, nlat, nlon) in C order (the Fortran (nlon, nlat, nlev)
grids), latitude north to south.

Parity pinning: the reference's own tests (tests/test_transport.f90:185-358)
hold no golden numbers, only invariants -- constancy of a uniform q under a
divergent wind, conservation of tracer mass, positivity, polar sub-stepping and
peak retention over one rotation -- and tests/test_transport_oracle.py checks
this restatement against each of them.  The operation order of every update
follows the reference line by line, so the CUDA path is compared against it at
round-off level.
"""
import numpy as np

R_EARTH = 6.371e6   # src/aeros_defs.f90:84
GRAV = 9.80665      # src/aeros_defs.f90:85
CFL_MAX = 0.9       # src/dynamics/aeros_transport.f90:144


class OracleTransport:
    """aeros_transport_class with its init (src/dynamics/aeros_transport.f90:155-203)."""

    def __init__(self, sinlat, gauss_w, nlon, a_half, b_half, vert_vanleer=False):
        self.nlat = len(sinlat)
        self.nlon = nlon
        self.A = np.asarray(a_half, dtype=np.float64)
        self.B = np.asarray(b_half, dtype=np.float64)
        self.nlev = len(self.A) - 1
        self.dlam = 2.0 * np.pi / nlon
        self.dmu = np.asarray(gauss_w, dtype=np.float64).copy()
        self.coslat = np.sqrt(np.maximum(0.0, 1.0 - np.asarray(sinlat) ** 2))
        cf = np.zeros(self.nlat + 1)
        muh = 1.0
        for j in range(self.nlat):
            muh = muh - self.dmu[j]
            cf[j + 1] = np.sqrt(max(0.0, 1.0 - muh * muh))
        cf[0] = 0.0
        cf[self.nlat] = 0.0
        self.cos_face = cf
        self.vert_vanleer = vert_vanleer
        self.last_cfl = 0.0
        self.last_nsub = 0

    # aeros_vgrid_pressure (src/dynamics/aeros_vertical.f90:344-380): layer thickness
    def _dp(self, ps):
        ph = self.A[:, None, None] + self.B[:, None, None] * ps[None]
        return ph[1:] - ph[:-1]

    def transport(self, u, v, lnps, q, dt):
        """aeros_transport_transport (:225-287); returns the new q."""
        ps = np.exp(lnps)
        self.dp_lev = self._dp(ps)
        self.qm = q * self.dp_lev
        cfl = self.max_courant(u, v, lnps, dt)
        nsub = max(1, int(np.ceil(cfl / CFL_MAX)))
        dts = dt / nsub
        self.last_cfl, self.last_nsub = cfl, nsub
        for _ in range(nsub):
            self._substep(u, v, dts)
        return self.qm / self.dp_lev

    def _substep(self, u, v, dt):
        """transport_substep (:289-372): zonal and meridional sweeps, then the
        vertical mass flux from the layer-mass change, updated top down in place."""
        dp0 = self.dp_lev.copy()
        self._sweep_zonal(u, dt)
        self._sweep_merid(v, dt)
        nlev = self.nlev
        scum = np.zeros((nlev + 1,) + dp0.shape[1:])
        for k in range(1, nlev + 1):
            scum[k] = scum[k - 1] + (dp0[k - 1] - self.dp_lev[k - 1]) / dt
        mfl = self.B[:, None, None] * scum[nlev][None] - scum
        qm, dpl = self.qm, self.dp_lev
        flux = self._vflux_vl if self.vert_vanleer else self._vflux
        for k in range(1, nlev + 1):            # Fortran level k = array index k - 1
            da = mfl[k] - mfl[k - 1]
            dq = flux(k, mfl[k], dt) - flux(k - 1, mfl[k - 1], dt)
            dpl[k - 1] = dpl[k - 1] - dt * da
            qm[k - 1] = qm[k - 1] - dt * dq

    # vflux_q (:596-630): donor cell through face k (between levels k and k + 1)
    def _vflux(self, k, mfl, dt):
        nlev = self.nlev
        if k <= 0 or k >= nlev:
            return np.zeros_like(mfl)
        qm, dpl = self.qm, self.dp_lev
        q_up = np.where(mfl >= 0.0, qm[k - 1] / dpl[k - 1], qm[k] / dpl[k])
        return q_up * mfl

    # vflux_q_vl (:632-688): van Leer through face k
    def _vflux_vl(self, k, mfl, dt):
        nlev = self.nlev
        if k <= 0 or k >= nlev:
            return np.zeros_like(mfl)
        qm, dpl = self.qm, self.dp_lev
        qa = lambda kk: qm[kk - 1] / dpl[kk - 1]
        down = mfl >= 0.0
        kd = np.where(down, k, k + 1)
        qd = np.where(down, qa(k), qa(k + 1))
        dpd = np.where(down, dpl[k - 1], dpl[k])
        cour = np.abs(mfl) * dt / dpd
        out = qd * mfl
        # downward: neighbours kd - 1 = k - 1, kd + 1 = k + 1; upward: kd + 1 = k + 2, kd - 1 = k
        ok_d = (k - 1 >= 1) and (k + 1 <= nlev)
        ok_u = (k + 2 <= nlev) and (k >= 1)
        res = out.copy()
        if ok_d:
            sm = qa(k) - qa(k - 1)
            sp = qa(k + 1) - qa(k)
            val = (qa(k) + 0.5 * (1.0 - cour) * _vanleer(sm, sp)) * mfl
            res = np.where(down, val, res)
        if ok_u:
            sm = qa(k + 1) - qa(k + 2)
            sp = qa(k) - qa(k + 1)
            val = (qa(k + 1) + 0.5 * (1.0 - cour) * _vanleer(sm, sp)) * mfl
            res = np.where(~down, val, res)
        return res

    def _sweep_zonal(self, u, dt):
        """sweep_zonal (:374-437): periodic van Leer fluxes at faces i + 1/2."""
        dc = self.dp_lev
        qc = self.qm / dc
        dx = (R_EARTH * self.coslat * self.dlam)[None, :, None]
        up = np.roll(u, -1, axis=2)
        uf = 0.5 * (u + up)
        cour = np.abs(uf) * dt / dx
        qm1, qp1, qp2 = np.roll(qc, 1, axis=2), np.roll(qc, -1, axis=2), np.roll(qc, -2, axis=2)
        # uf >= 0: upwind cell i, dir +1: sm = q(i) - q(i-1), sp = q(i+1) - q(i)
        qf_p = qc + 0.5 * (1.0 - cour) * _vanleer(qc - qm1, qp1 - qc)
        # uf < 0: upwind cell i+1, dir -1: sm = q(i+1) - q(i+2), sp = q(i) - q(i+1)
        qf_m = qp1 + 0.5 * (1.0 - cour) * _vanleer(qp1 - qp2, qc - qp1)
        pos = uf >= 0.0
        fair = np.where(pos, dc * uf, np.roll(dc, -1, axis=2) * uf)
        fq = np.where(pos, qf_p, qf_m) * fair
        fair_m, fq_m = np.roll(fair, 1, axis=2), np.roll(fq, 1, axis=2)
        self.dp_lev = self.dp_lev - dt * (fair - fair_m) / dx
        self.qm = self.qm - dt * (fq - fq_m) / dx

    def _sweep_merid(self, v, dt):
        """sweep_merid (:439-503): van Leer fluxes at faces j + 1/2, zero at the poles."""
        nlat = self.nlat
        dc = self.dp_lev
        qc = self.qm / dc
        fair = np.zeros((self.nlev, nlat + 1, self.nlon))
        fq = np.zeros_like(fair)
        for j in range(1, nlat):                # face between Fortran rows j and j + 1
            jj = j - 1                          # 0-based row j
            vf = 0.5 * (v[:, jj] + v[:, jj + 1])
            dy = R_EARTH * self.dmu[jj] / max(self.cos_face[j], 1.0e-6)
            cour = np.abs(vf) * dt / dy
            qf_p = self._vl_bounded(qc, j, +1, cour)
            qf_m = self._vl_bounded(qc, j + 1, -1, cour)
            pos = vf >= 0.0
            fa = np.where(pos, dc[:, jj] * vf * self.cos_face[j], dc[:, jj + 1] * vf * self.cos_face[j])
            fair[:, j] = fa
            fq[:, j] = np.where(pos, qf_p, qf_m) * fa
        den = (R_EARTH * self.dmu)[None, :, None]
        self.dp_lev = self.dp_lev - dt * (fair[:, 1:] - fair[:, :-1]) / den
        self.qm = self.qm - dt * (fq[:, 1:] - fq[:, :-1]) / den

    def _vl_bounded(self, qc, jup, d, cour):
        """vl_face_bounded (:542-573), Fortran row jup."""
        n = self.nlat
        q = lambda jf: qc[:, jf - 1]
        if jup <= 1 or jup >= n:
            return q(jup)
        if d > 0:
            sm, sp = q(jup) - q(jup - 1), q(jup + 1) - q(jup)
        else:
            sm, sp = q(jup) - q(jup + 1), q(jup - 1) - q(jup)
        return q(jup) + 0.5 * (1.0 - cour) * _vanleer(sm, sp)

    def max_courant(self, u, v, lnps, dt):
        """max_courant (:690-741)."""
        dpc = self._dp(np.exp(lnps))
        dxc = (R_EARTH * self.coslat * self.dlam)[None, :, None]
        cmass = dpc * np.abs(u) / dxc
        scum = np.zeros((self.nlev + 1,) + dpc.shape[1:])
        for k in range(1, self.nlev + 1):
            scum[k] = scum[k - 1] + cmass[k - 1]
        dy = (R_EARTH * self.dmu / np.maximum(self.coslat, 1.0e-6))[None, :, None]
        cx = np.abs(u) * dt / dxc
        cy = np.abs(v) * dt / dy
        B = self.B[:, None, None]
        cz = (np.abs(B[1:] * scum[-1][None] - scum[1:]) + np.abs(B[:-1] * scum[-1][None] - scum[:-1])) * dt / dpc
        return float(np.max(cx + cy + cz))

    def water(self, ps, q):
        """aeros_transport_water (:743-779): total tracer mass [kg]."""
        dpc = self._dp(ps)
        col = np.zeros(ps.shape)
        for k in range(self.nlev):
            col = col + q[k] * dpc[k]
        area = self.dmu * (2.0 * np.pi / self.nlon) * R_EARTH * R_EARTH   # src/aeros_grid.f90:71-77
        tot = 0.0
        for j in range(self.nlat):
            for i in range(self.nlon):
                tot = tot + col[j, i] * area[j] / GRAV
        return tot


def _vanleer(a, b):
    """vanleer (:575-594): harmonic-mean slope, 0 at an extremum."""
    ab = a * b
    with np.errstate(divide="ignore", invalid="ignore"):
        s = 2.0 * a * b / (a + b)
    return np.where(ab > 0.0, s, 0.0)
