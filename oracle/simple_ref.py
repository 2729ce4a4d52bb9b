"""The isothermal SIMPLE outer iteration of the reference (src/Simple.f:
299-660) driven through the oracle's restated cell routines
(fvc_oracle_simple.c) and solvers (fvc_oracle.c).

TEST INFRASTRUCTURE ONLY: the checker of the GPU SIMPLE loop and the CPU
leg of its benchmark; the product never imports this module.  A case is a
dict with coor (nnode,2), ix (numel,nshared+1, material last), nelcon,
num, ident (numeq), pedge (numel,nshared+1), sedge (numel,nshared+1,3),
e (nmat,10), nshared and numel (fortranfvcell_gb300.cases builds one).
"""
import numpy as np


class SimpleRef:
    """One reference SIMPLE state advanced by the oracle.  Defaults follow
    the C1 configuration: u, v BiCGSTAB on ELLPACK, p' PCG on CSRD, steady
    (large dt), no second-order time term, SIMPLE (not SIMPLEC)."""

    def __init__(self, orc, case, dt=1.0e10, under_u=0.7, under_pc=0.3, simple_c=False,
                 tol_pcg=1e-8, tol_bcg=1e-8, maxit=50000, matriz_u=4, matriz_pc=1,
                 int_vel=5):
        self.orc, self.m = orc, case
        self.dt, self.under_u, self.under_pc, self.simple_c = dt, under_u, under_pc, simple_c
        self.tol_pcg, self.tol_bcg, self.maxit = tol_pcg, tol_bcg, maxit
        self.mu, self.mpc, self.int_vel = matriz_u, matriz_pc, int_vel
        n = case["numel"]
        self.n = n
        self.iau, self.jau, self.nadu = orc.datastruc(case["ident"], matriz_u, True)
        self.iapc, self.japc, self.nadpc = orc.datastruc(case["ident"], matriz_pc, True)
        z2 = lambda: np.zeros((n, 2))
        self.w, self.gu1, self.gu2, self.gp, self.gpc, self.d = z2(), z2(), z2(), z2(), z2(), z2()
        self.im = np.zeros((n, 4))
        self.p, self.pc = np.zeros(n), np.zeros(n)
        self.u1, self.u2 = np.zeros(n), np.zeros(n)
        self.it = 0
        self.r0 = {}
        self.history = []
        # time term F = rho cc A/dt u (before the loop, Simple.f:247-266)
        self.b10, self.b20 = np.zeros(n), np.zeros(n)
        for comp, b0 in ((1, self.b10), (2, self.b20)):
            u = self.w[:, comp - 1].copy()
            orc.pform_momentum(case, comp, 3, u, u, self.w, self.gu1, self.gu2, self.gp, dt,
                               self.iau, self.jau, matriz_u, b0, self.im, self.d,
                               np.zeros(n), bs=False, under_u=under_u, simple_c=simple_c)

    def _nnz(self, matriz, ja):
        return ja.size

    def _momentum(self, comp):
        orc, m, n = self.orc, self.m, self.n
        u = self.u1 if comp == 1 else self.u2
        g_own, g_oth = (self.gu1, self.gu2) if comp == 1 else (self.gu2, self.gu1)
        ad = np.zeros(n)
        au = np.zeros(self.jau.size)
        b = np.zeros(n)
        rc = np.zeros(n)
        orc.pform_momentum(m, comp, 1, u, self.p, self.w, g_own, g_oth, self.gp, self.dt,
                           self.iau, self.jau, self.mu, b, self.im, self.d, rc, ad=ad, au=au,
                           bs=False, under_u=self.under_u, simple_c=self.simple_c)
        b0 = self.b10 if comp == 1 else self.b20
        b = b + b0                                      # asumb
        sx = np.zeros(n)
        orc.lib().oref_getres(orc._p(sx), orc._p(b0), orc._p(m["num"]), n, n, 0)
        rc = rc + sx
        return ad, au, b, rc

    def _solve(self, ad, au, b, x_cells, code, matriz, ia, ja, nad, tol):
        orc, m, n = self.orc, self.m, self.n
        sx = np.zeros(n)
        orc.lib().oref_getres(orc._p(np.ascontiguousarray(x_cells)), orc._p(sx),
                              orc._p(m["num"]), n, n, 1)
        # the solver overwrites b (as p or s, src/Iterativos.f); the system
        # stays as assembled for whoever inspects it afterwards
        st = orc.solver(ad, au, au, sx, b.copy(), ia, ja, n, nad, True, tol, self.maxit, code,
                        matriz)
        out = np.zeros(n)
        orc.lib().oref_getres(orc._p(out), orc._p(sx), orc._p(m["num"]), n, n, 0)
        return out, st

    def step(self):
        """One outer iteration; returns (rU1, rU2, rPc) as Simple.f computes
        them (cell-residual 2-norms)."""
        orc, m, n = self.orc, self.m, self.n
        self.it += 1
        self.u1, self.u2 = self.w[:, 0].copy(), self.w[:, 1].copy()          # guess
        orc.gform(m, 1, 1, self.u1, self.gu1)
        orc.gform(m, 1, 2, self.u2, self.gu2)
        self.div = orc.divergente(self.gu1, self.gu2)
        orc.gform(m, 2, 3, self.p, self.gp)
        ad1, au1, b1, rc1 = self._momentum(1)
        ad2, au2, b2, rc2 = self._momentum(2)
        # a momentum equation whose right-hand side vanishes is not solved
        # (Simple.f:437-441, 462-466: b.b < 1e-32)
        self.solved = (float(b1 @ b1) >= 1.0e-32, float(b2 @ b2) >= 1.0e-32)
        if self.solved[0]:
            self.u1, self.st_u1 = self._solve(ad1, au1, b1, self.u1, 2, self.mu, self.iau,
                                              self.jau, self.nadu, self.tol_bcg)
        if self.solved[1]:
            self.u2, self.st_u2 = self._solve(ad2, au2, b2, self.u2, 2, self.mu, self.iau,
                                              self.jau, self.nadu, self.tol_bcg)
        wp = np.stack([self.u1, self.u2], axis=1)                            # updateVel
        adp, aup, bp, rcp = np.zeros(n), np.zeros(self.japc.size), np.zeros(n), np.zeros(n)
        orc.pform_pc(m, wp, self.d, self.p, self.gp, self.iapc, self.japc, self.mpc, adp, aup,
                     bp, rcp, int_vel=self.int_vel)
        self.systems = dict(u1=(ad1, au1, b1), u2=(ad2, au2, b2), pc=(adp, aup, bp))
        r_pc = float(np.sqrt(rcp @ rcp))
        r_u1 = float(np.sqrt(rc1 @ rc1))
        r_u2 = float(np.sqrt(rc2 @ rc2))
        if self.it == 1:
            self.r0 = dict(pc=r_pc, u1=r_u1, u2=r_u2)
        if r_pc >= 1.0e-32:
            self.pc, self.st_pc = self._solve(adp, aup, bp, self.pc, 1, self.mpc, self.iapc,
                                              self.japc, self.nadpc, self.tol_pcg)
            orc.gform(m, 2, 2, self.pc, self.gpc)
            orc.simple_update(self.w, self.p, self.u1, self.u2, self.pc, self.gpc, self.d,
                              self.under_pc)
        self.history.append((r_u1, r_u2, r_pc))
        return r_u1, r_u2, r_pc


class GasSimpleRef(SimpleRef):
    """The ideal-gas SIMPLE iteration with the energy equation (materials of
    type 53/55; src/Simple.f:229-300, 299-845 with sEnergy; start-up of
    src/Main.f:815-837): momentum cell_si_eb_idg_ggl with buoyancy, p'
    cell_si_p_idg_ggl, enthalpy cell_e_eb_idg_ggl (lib 3, CSRD, BiCGSTAB),
    then T from the enthalpy and the density row 3 from the ideal-gas law;
    time steps shift the density levels (massUpdate).  The case also holds
    pedgeE / sedgeE (numel, nshared+1), gravity (2,) and the initial
    temperature t0.  The domain is open (cPc0/cPc = 1: no closedPresure)."""

    def __init__(self, orc, case, dt=0.02, bs=False, tol_e=None, t0=20.0, **kw):
        super().__init__(orc, case, dt=dt, **kw)
        n = self.n
        self.bs = bs
        self.tol_e = self.tol_bcg if tol_e is None else tol_e
        self.grav = np.asarray(case["gravity"], np.float64)
        self.pe, self.se = case["pedgeE"], case["sedgeE"]
        self.iae, self.jae, self.nade = orc.datastruc(case["ident"], 1, True)
        e = case["e"]
        self.cp, self.tref = e[0, 3], e[0, 4]
        self.temp = np.full(n, float(t0))
        self.en = np.zeros(n)
        orc.enthalpy_temp(self.en, self.temp, e, False)
        self.en0 = self.en.copy()
        self.ro = np.zeros((n, 3))
        for row in (1, 2, 3):
            orc.ideal_gas(self.ro, self.temp, row)
        self.ge = np.zeros((n, 2))
        self.w0 = self.w.copy()
        self.div = np.zeros(n)
        self.start_step()

    def start_step(self):
        """Time terms of a new step (Simple.f:229-300): momentum from the
        densities of levels n-1, n, w0 = w; the enthalpy's with its source;
        en0 = en."""
        orc, m, n = self.orc, self.m, self.n
        for comp, b0 in ((1, self.b10), (2, self.b20)):
            b0[:] = 0.0
            u, u0 = self.w[:, comp - 1].copy(), self.w0[:, comp - 1].copy()
            orc.pform_momentum_idg(m, comp, 3, u, u0, self.w, self.gu1, self.gu2, self.gp,
                                   self.ro, self.div, self.grav, self.dt, self.iau, self.jau,
                                   self.mu, b0, self.im, self.d, np.zeros(n), bs=self.bs,
                                   under_u=self.under_u, simple_c=self.simple_c)
        self.w0 = self.w.copy()
        self.bE0 = np.zeros(n)
        orc.pform_energy(m, 3, 4, self.pe, self.se, self.en, self.en0, self.ro, self.w, self.ge,
                         self.dt, self.iae, self.jae, 1, self.bE0, np.zeros(n), bs=self.bs)
        self.en0 = self.en.copy()

    def end_step(self):
        """massUpdate (Simple.f:1041-1050): ro(1) = ro(2), ro(2) = ro(3)."""
        self.ro[:, 0] = self.ro[:, 1]
        self.ro[:, 1] = self.ro[:, 2]

    def _momentum(self, comp):
        orc, m, n = self.orc, self.m, self.n
        u = self.u1 if comp == 1 else self.u2
        g_own, g_oth = (self.gu1, self.gu2) if comp == 1 else (self.gu2, self.gu1)
        ad, au, b, rc = np.zeros(n), np.zeros(self.jau.size), np.zeros(n), np.zeros(n)
        orc.pform_momentum_idg(m, comp, 1, u, self.p, self.w, g_own, g_oth, self.gp, self.ro,
                               self.div, self.grav, self.dt, self.iau, self.jau, self.mu, b,
                               self.im, self.d, rc, ad=ad, au=au, bs=self.bs,
                               under_u=self.under_u, simple_c=self.simple_c)
        b0 = self.b10 if comp == 1 else self.b20
        b = b + b0
        sx = np.zeros(n)
        orc.lib().oref_getres(orc._p(sx), orc._p(b0), orc._p(m["num"]), n, n, 0)
        return ad, au, b, rc + sx

    def step(self):
        """One outer iteration; returns (rU1, rU2, rPc, rE)."""
        orc, m, n = self.orc, self.m, self.n
        self.it += 1
        self.u1, self.u2 = self.w[:, 0].copy(), self.w[:, 1].copy()
        orc.gform(m, 1, 1, self.u1, self.gu1)
        orc.gform(m, 1, 2, self.u2, self.gu2)
        self.div = orc.divergente(self.gu1, self.gu2)
        orc.gform(m, 3, 3, self.p, self.gp)
        ad1, au1, b1, rc1 = self._momentum(1)
        ad2, au2, b2, rc2 = self._momentum(2)
        self.solved = (float(b1 @ b1) >= 1.0e-32, float(b2 @ b2) >= 1.0e-32)
        if self.solved[0]:
            self.u1, self.st_u1 = self._solve(ad1, au1, b1, self.u1, 2, self.mu, self.iau,
                                              self.jau, self.nadu, self.tol_bcg)
        if self.solved[1]:
            self.u2, self.st_u2 = self._solve(ad2, au2, b2, self.u2, 2, self.mu, self.iau,
                                              self.jau, self.nadu, self.tol_bcg)
        wp = np.stack([self.u1, self.u2], axis=1)
        adp, aup, bp, rcp = np.zeros(n), np.zeros(self.japc.size), np.zeros(n), np.zeros(n)
        orc.pform_pc_idg(m, wp, self.d, self.p, self.gp, self.ro, self.dt, self.iapc, self.japc,
                         self.mpc, adp, aup, bp, rcp, int_vel=self.int_vel, bs=self.bs)
        r_pc = float(np.sqrt(rcp @ rcp))
        r_u1 = float(np.sqrt(rc1 @ rc1))
        r_u2 = float(np.sqrt(rc2 @ rc2))
        if r_pc >= 1.0e-32:
            self.pc, self.st_pc = self._solve(adp, aup, bp, self.pc, 1, self.mpc, self.iapc,
                                              self.japc, self.nadpc, self.tol_pcg)
            orc.gform(m, 3, 2, self.pc, self.gpc)
            orc.simple_update(self.w, self.p, self.u1, self.u2, self.pc, self.gpc, self.d,
                              self.under_pc)
        # energy (Simple.f:647-710)
        orc.gform_energy(m, 3, self.pe, self.se, self.en, self.ge)
        ade, aue, be, rce = np.zeros(n), np.zeros(self.jae.size), np.zeros(n), np.zeros(n)
        orc.pform_energy(m, 3, 1, self.pe, self.se, self.en, self.en, self.ro, self.w, self.ge,
                         self.dt, self.iae, self.jae, 1, be, rce, ad=ade, au=aue, bs=self.bs)
        be = be + self.bE0
        sx = np.zeros(n)
        orc.lib().oref_getres(orc._p(sx), orc._p(self.bE0), orc._p(m["num"]), n, n, 0)
        rce = rce + sx
        r_e = float(np.sqrt(be @ be))
        self.solved_e = r_e >= 1.0e-32
        if self.solved_e:
            r_e = float(np.sqrt(rce @ rce))
            self.en, self.st_e = self._solve(ade, aue, be, self.en, 2, 1, self.iae, self.jae,
                                             self.nade, self.tol_e)
            orc.enthalpy_temp(self.en, self.temp, m["e"], True)
            orc.ideal_gas(self.ro, self.temp, 3)
        self.history.append((r_u1, r_u2, r_pc, r_e))
        return r_u1, r_u2, r_pc, r_e
