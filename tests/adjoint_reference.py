"""Host restatement of the MCTDHF pulse-gradient adjoint (numpy, FP64).

TEST INFRASTRUCTURE ONLY: the reference the GPU adjoint
(cgpu_mc_adjoint_forward / cgpu_mc_adjoint_backward) is compared against.

Systems: restricted MCTDHF with two body types of one particle each.  The
configuration space is the M x M coefficient matrix C (index a + M b); the
NonLin derivative of the reference (src/Method/Mb/OrbBased/Mctdhx/S_Method_Mb_OrbBased_Mctdhx.f90:180-226,
ApplyCorrelationOp src/Method/Mb/OrbBased/S_Method_Mb_OrbBased.f90:647-805,
Coeffs_Generic src/Coeffs/Generic/S_Coeffs_Generic.f90:103-319) in dense form:
  dC = -i P_C (h1^T C + C h1 + sum_ab g(a,b;c,d) C_ab),
  dphi = -i (1 - P) sum W_lk phi_a R[a,k,j,l],  R = rho2 . U n/(n^2+eps) U^H.
`Dense.forward` is checked against the oracle's NonLin derivative and
`Dense.vjp` against finite differences in tests/test_adjoint_reference.py.
`Adjoint` differentiates the Strang step SIL(OrbsLin, dt/2) -> RK4(NonLin, dt)
-> SIL(OrbsLin, dt/2) with the field E(t) = field[floor(t / dt)] and the
objective J = 1 - |<Psi_ref|Psi_N>|^2, with checkpointing.
"""
import numpy as np

class Dense:
    def __init__(self, o, Vint):
        self.o, self.V = o, Vint
        self.nG, self.M = o.nG, o.nOS
        self.w = o.w; self.x = o.x
        self.eps = o.spec.reg_eps
        # kinetic as a dense matrix A0 (columns = kinetic_apply of unit vectors) + V0
        nG = self.nG
        A = np.zeros((nG, nG))
        for j in range(nG):
            e = np.zeros(nG, complex); e[j] = 1.0
            A[:, j] = o.kinetic_apply(e, 0).real
        self.A0 = A + np.diag(o.potential())
    def A(self, E):
        return self.A0 + np.diag(E*self.x)
    def unpack(self, st):
        M, nG = self.M, self.nG
        return st[:M*M].reshape(M, M).T.copy(), st[M*M:].reshape(M, nG).T.copy()
    def pack(self, C, phi):
        return np.concatenate([C.T.reshape(-1), phi.T.reshape(-1)])
    def forward(self, st, E):
        C, phi = self.unpack(st)
        w, V, eps = self.w, self.V, self.eps
        A = self.A(E)
        Aphi = A @ phi
        h1 = phi.conj().T @ (w[:,None]*Aphi)
        Sp = np.einsum('yb,yd,y->ybd', phi.conj(), phi, w)
        Wp = np.einsum('xy,ybd->xbd', V, Sp)
        g = np.einsum('xa,xbd,xc,x->abcd', phi.conj(), Wp, phi, w)
        dC0 = h1.T @ C + C @ h1 + np.einsum('abcd,ab->cd', g, C)
        r1 = np.conj(C) @ C.T + C.conj().T @ C
        r2 = np.einsum('cd,ab->abcd', C, C.conj()) + np.einsum('dc,ba->abcd', C, C.conj())
        occ, U = np.linalg.eigh(r1)
        f = occ/(occ**2 + eps)
        Mreg = (U*f) @ U.conj().T
        R = np.einsum('abkd,kj->abjd', r2, Mreg)
        dphi0 = np.einsum('xlk,xa,akjl->xj', Wp, phi, R)
        c = C.T.reshape(-1); d = dC0.T.reshape(-1)
        s = c.conj() @ d
        dCv = d - s*c
        Gp = phi.conj().T @ (w[:,None]*dphi0)
        dphi = dphi0 - phi @ Gp
        tape = dict(C=C, phi=phi, A=A, Aphi=Aphi, h1=h1, Sp=Sp, Wp=Wp, g=g, dC0=dC0, r1=r1, r2=r2, occ=occ, U=U, f=f,
                    Mreg=Mreg, R=R, dphi0=dphi0, s=s, Gp=Gp)
        out = -1j*np.concatenate([dCv, dphi.T.reshape(-1)])
        return out, tape
    def vjp(self, tape, obar):
        M, nG, w, V, eps = self.M, self.nG, self.w, self.V, self.eps
        T = tape
        C, phi = T['C'], T['phi']
        ubar = 1j*obar       # y = -i u
        dCv_bar = ubar[:M*M]; dphi_bar = ubar[M*M:].reshape(M, nG).T
        c = C.T.reshape(-1); d = T['dC0'].T.reshape(-1)
        # C projection
        d_bar = dCv_bar - c*(c.conj() @ dCv_bar)
        c_bar = -np.conj(T['s'])*dCv_bar - (dCv_bar.conj() @ c)*d
        Cbar = c_bar.reshape(M, M).T.copy()
        dC0_bar = d_bar.reshape(M, M).T
        # phi projection
        Wd = w[:,None]*T['dphi0']
        dphi0_bar = dphi_bar - (w[:,None]*phi) @ (phi.conj().T @ dphi_bar)
        phibar = -dphi_bar @ T['Gp'].conj().T - Wd @ (dphi_bar.conj().T @ phi)
        # dC0 = h1^T C + C h1 + G
        h1 = T['h1']
        Cbar += np.conj(h1) @ dC0_bar + dC0_bar @ h1.conj().T
        h1bar = np.conj(C) @ dC0_bar.T + C.conj().T @ dC0_bar
        Cbar += np.einsum('abcd,cd->ab', T['g'].conj(), dC0_bar)
        gbar = np.einsum('cd,ab->abcd', dC0_bar, C.conj())
        # h1 = phi^H W A phi
        X1 = phi.conj().T @ (w[:,None]*(self.x[:,None]*phi))
        Ebar = np.real(np.sum(np.conj(h1bar)*X1))
        phibar += w[:,None]*(T['Aphi'] @ h1bar.conj().T) + w[:,None]*(T['A'] @ (phi @ h1bar))
        # g = sum_x conj(phi_a) Wp_bd phi_c w
        Wp = T['Wp']
        phibar += w[:,None]*np.einsum('abcd,xbd,xc->xa', gbar.conj(), Wp, phi)
        phibar += w[:,None]*np.einsum('abcd,xa,xbd->xc', gbar, phi, Wp.conj())
        Wpbar = w[:,None,None]*np.einsum('abcd,xa,xc->xbd', gbar, phi, phi.conj())
        # dphi0 = sum Wp[x,l,k] phi[x,a] R[a,k,j,l]
        R = T['R']
        Rbar = np.einsum('xlk,xa,xj->akjl', Wp.conj(), phi.conj(), dphi0_bar)
        Wpbar += np.einsum('xa,akjl,xj->xlk', phi.conj(), R.conj(), dphi0_bar)
        phibar += np.einsum('xlk,akjl,xj->xa', Wp.conj(), R.conj(), dphi0_bar)
        # R = r2 . Mreg
        r2bar = np.einsum('abjd,kj->abkd', Rbar, T['Mreg'].conj())
        Mbar = np.einsum('abkd,abjd->kj', T['r2'].conj(), Rbar)
        # Mreg = U f U^H
        occ, U, f = T['occ'], T['U'], T['f']
        dn = occ[:,None] - occ[None,:]
        fp = (eps - occ**2)/(occ**2 + eps)**2
        with np.errstate(divide='ignore', invalid='ignore'):
            F = np.where(np.abs(dn) > 1e-13*np.maximum(1.0, np.abs(occ[:,None])), (f[:,None]-f[None,:])/dn, 0.5*(fp[:,None]+fp[None,:]))
        r1bar = U @ (F*(U.conj().T @ Mbar @ U)) @ U.conj().T
        # r1 = conj(C) C^T + C^H C
        Cbar += r1bar.T @ C + np.conj(r1bar) @ C + C @ r1bar + C @ r1bar.conj().T
        # r2 = C_cd conj(C_ab) + C_dc conj(C_ba)
        Cbar += np.einsum('abcd,ab->cd', r2bar, C) + np.einsum('abcd,cd->ab', r2bar.conj(), C)
        Cbar += np.einsum('abcd,ba->dc', r2bar, C) + np.einsum('abcd,dc->ba', r2bar.conj(), C)
        # Wp = V Sp, Sp = conj(phi_b) phi_d w
        Spbar = np.einsum('xy,xbd->ybd', V, Wpbar)
        phibar += np.einsum('ybd,yb,y->yd', Spbar, phi, w)
        phibar += np.einsum('ybd,yd,y->yb', Spbar.conj(), phi, w)
        return self.pack(Cbar, phibar), Ebar


def mdot(a, b, m):
    return np.sum(np.conj(a) * m * b)


class Adjoint:
    """Dense reference of the pulse-gradient adjoint for (1,1)-restricted MCTDHF:
    Strang step = SIL(OrbsLin, dt/2) -> RK4(NonLin, dt) -> SIL(OrbsLin, dt/2), field sampled per step."""

    def __init__(self, D, field, dt, K):
        self.D, self.field, self.dt, self.K = D, np.asarray(field, float), dt, K
        M, nG = D.M, D.nG
        self.m = np.concatenate([np.ones(M * M), np.tile(D.w, M)])
        self.X = np.concatenate([np.zeros(M * M), np.tile(D.x, M)])

    def E(self, t):
        n = int(np.floor(t / self.dt + 1e-9))
        return (self.field[n] if 0 <= n < len(self.field) else 0.0), n

    def H(self, v, E):
        M, nG = self.D.M, self.D.nG
        out = np.zeros_like(v)
        phi = v[M * M:].reshape(M, nG).T
        out[M * M:] = (self.D.A(E) @ phi).T.reshape(-1)
        return out

    def HT(self, v, E):
        M, nG = self.D.M, self.D.nG
        out = np.zeros_like(v)
        phi = v[M * M:].reshape(M, nG).T
        out[M * M:] = (self.D.A(E).T @ phi).T.reshape(-1)
        return out

    def lanczos(self, s, E, tau):
        K, m = self.K, self.m
        n0 = np.sqrt(mdot(s, s, m).real)
        V = [s / n0]
        al, be = [], []
        for j in range(K):
            w = self.H(V[j], E)
            if j > 0:
                w = w - be[j - 1] * V[j - 1]
            a = mdot(V[j], w, m).real
            w = w - a * V[j]
            for k in range(j + 1):
                w = w - mdot(V[k], w, m) * V[k]
            al.append(a)
            b = np.sqrt(mdot(w, w, m).real)
            be.append(b)
            if j < K - 1:
                V.append(w / b)
        T = np.diag(al) + np.diag(be[:K - 1], 1) + np.diag(be[:K - 1], -1)
        lam, Q = np.linalg.eigh(T)
        y = Q @ (np.exp(-1j * tau * lam) * Q[0, :])
        out = n0 * np.array(V).T @ y
        return out, dict(n0=n0, V=V, al=al, be=be, lam=lam, Q=Q, y=y, tau=tau, s=s, E=E)

    def lanczos_vjp(self, tp, obar):
        K, m = self.K, self.m
        V, al, be, lam, Q, y, tau, n0, E = tp['V'], tp['al'], tp['be'], tp['lam'], tp['Q'], tp['y'], tp['tau'], tp['n0'], tp['E']
        Vm = np.array(V).T
        n0bar = np.real(np.vdot(Vm @ y, obar))
        vbar = [n0 * np.conj(y[j]) * obar for j in range(K)]
        ybar = n0 * (Vm.conj().T @ obar)
        # Frechet adjoint of exp(-i tau T) e1
        e = np.exp(-1j * tau * lam)
        dl = lam[:, None] - lam[None, :]
        with np.errstate(divide='ignore', invalid='ignore'):
            F = np.where(np.abs(dl) > 1e-12, (e[:, None] - e[None, :]) / dl, -1j * tau * e[:, None] * np.ones_like(dl))
        a = Q.T @ ybar
        q = Q[0, :]
        Bbar = np.real(np.conj(a)[:, None] * F * q[None, :])
        Tbar = Q @ Bbar @ Q.T
        abar = [Tbar[j, j] for j in range(K)]
        bbar = [Tbar[j, j + 1] + Tbar[j + 1, j] for j in range(K - 1)] + [0.0]
        Ebar = 0.0
        # the three-term recurrence in reverse (the re-orthogonalisation is the identity in exact arithmetic)
        rj = [None] * K
        for j in range(K):
            w = self.H(V[j], E) - (be[j - 1] * V[j - 1] if j > 0 else 0)
            rj[j] = w - al[j] * V[j]
        for j in range(K - 1, -1, -1):
            r = rj[j]
            rbar = np.zeros_like(r)
            if j < K - 1:
                rbar += vbar[j + 1] / be[j]
                bbar[j] += -np.real(np.vdot(vbar[j + 1], r)) / be[j] ** 2
                rbar += bbar[j] * (m * r) / be[j]
            wbar = rbar.copy()
            abar[j] += -np.real(np.vdot(rbar, V[j]))
            vbar[j] = vbar[j] - al[j] * rbar
            w = r + al[j] * V[j]
            wbar += abar[j] * (m * V[j])
            vbar[j] = vbar[j] + abar[j] * (m * w)
            vbar[j] = vbar[j] + self.HT(wbar, E)
            Ebar += np.real(np.vdot(wbar, self.X * V[j]))
            if j > 0:
                bbar[j - 1] += -np.real(np.vdot(wbar, V[j - 1]))
                vbar[j - 1] = vbar[j - 1] - be[j - 1] * wbar
        s = tp['s']
        sbar = vbar[0] / n0
        n0bar += -np.real(np.vdot(vbar[0], s)) / n0 ** 2
        sbar = sbar + n0bar * (m * s) / n0
        return sbar, Ebar

    def rk4(self, s, t0):
        dt = self.dt
        D = self.D
        E1, n1 = self.E(t0); E2, n2 = self.E(t0 + dt / 2); E4, n4 = self.E(t0 + dt)
        k1, t1 = D.forward(s, E1)
        s2 = s + dt / 2 * k1; k2, t2 = D.forward(s2, E2)
        s3 = s + dt / 2 * k2; k3, t3 = D.forward(s3, E2)
        s4 = s + dt * k3; k4, t4 = D.forward(s4, E4)
        out = s + dt / 6 * k1 + dt / 3 * k2 + dt / 3 * k3 + dt / 6 * k4
        return out, [(t1, n1), (t2, n2), (t3, n2), (t4, n4)]

    def rk4_vjp(self, tapes, obar, grad):
        dt = self.dt
        sbar = obar.copy()
        kb = [dt / 6 * obar, dt / 3 * obar, dt / 3 * obar, dt / 6 * obar]
        for i, coef in ((3, dt), (2, dt / 2), (1, dt / 2), (0, None)):
            tp, n = tapes[i]
            sb, eb = self.D.vjp(tp, kb[i])
            if 0 <= n < len(grad):
                grad[n] += eb
            sbar += sb
            if coef is not None:
                kb[i - 1] = kb[i - 1] + coef * sb
        return sbar

    def step(self, s, n):
        dt = self.dt
        t0 = n * dt
        Ea, na = self.E(t0 + dt / 4)
        a, la = self.lanczos(s, Ea, dt / 2)
        b, tb = self.rk4(a, t0)
        Ec, nc = self.E(t0 + dt / 2 + dt / 4)
        c, lc = self.lanczos(b, Ec, dt / 2)
        return c, (la, na, tb, lc, nc)

    def step_vjp(self, tape, obar, grad):
        la, na, tb, lc, nc = tape
        bbar, e = self.lanczos_vjp(lc, obar); grad[nc] += e
        abar = self.rk4_vjp(tb, bbar, grad)
        sbar, e = self.lanczos_vjp(la, abar); grad[na] += e
        return sbar

    def overlap(self, s0, s):
        D = self.D
        C0, f0 = D.unpack(s0); C, f = D.unpack(s)
        S = f0.conj().T @ (D.w[:, None] * f)
        return np.sum(np.conj(C0) * (S @ C @ S.T)), S

    def run(self, s0, checkpoint=4):
        D = self.D
        N = len(self.field)
        chk = {}
        s = s0.copy()
        for n in range(N):
            if n % checkpoint == 0:
                chk[n] = s.copy()
            s, _ = self.step(s, n)
        O, S = self.overlap(s0, s)
        J = 1.0 - abs(O) ** 2
        # objective gradient w.r.t. the final state
        Ob = -2.0 * O
        C0, f0 = D.unpack(s0); C, f = D.unpack(s)
        Cb = Ob * (S.conj().T @ C0 @ S.conj())
        P = np.conj(C0)
        Sb = Ob * np.conj(P @ S @ C.T + P.T @ S @ C)
        fb = D.w[:, None] * (f0 @ Sb)
        lam = D.pack(Cb, fb)
        grad = np.zeros(N)
        for seg in sorted(chk.keys(), reverse=True):
            states = [chk[seg]]
            tapes = []
            for n in range(seg, min(seg + checkpoint, N)):
                nxt, tp = self.step(states[-1], n)
                states.append(nxt); tapes.append(tp)
            for i in range(len(tapes) - 1, -1, -1):
                lam = self.step_vjp(tapes[i], lam, grad)
        return J, O, s, grad
