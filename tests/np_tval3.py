"""Independent numpy restatement of the reference TVAL3 loop (3d/tval3_gpu_3d.cpp:1089-1345),
written separately from oracle/tval3_oracle.cpp and used by the tests to pin
that oracle (same control flow, same result).  Test helper only.
"""
import numpy as np
import scipy.sparse as sp

def Dop(U, dims):
    p,q,r = dims; V = U.reshape(r,q,p)
    return np.stack([np.roll(V,-1,axis=2)-V, np.roll(V,-1,axis=1)-V, np.roll(V,-1,axis=0)-V]).reshape(3,-1)
def Dtop(X, dims):
    p,q,r = dims; X = X.reshape(3,r,q,p)
    return ((np.roll(X[0],1,axis=2)-X[0]) + (np.roll(X[1],1,axis=1)-X[1]) + (np.roll(X[2],1,axis=0)-X[2])).reshape(-1)

def tval3(A, b, dims, o, iso=False):
    m, n = A.shape
    bmin = b[np.argmin(np.abs(b))]; bmax = b[np.argmax(np.abs(b))]; dif = abs(bmax-bmin)
    scl = 0.5/dif if dif < 0.5 else (1.5/dif if dif > 1.5 else 1.0)
    b = b*scl
    At = A.T.tocsr()
    Atb = At@b; U = Atb.copy()
    mu, beta = min(o['mu0'],o['mu']), min(o['beta0'],o['beta']); gam = o['gam']
    sig = np.zeros((3,n)); delta = np.zeros(m); DtsAtd = np.zeros(n)
    st = {}
    def shrink(DU):
        ub = DU - sig/beta
        if not iso:
            t = np.maximum(np.abs(ub)-1/beta,0); W_ = np.sign(ub)*t; W_[ub>=0] = t[ub>=0]; W_[ub<0] = -t[ub<0]; return W_, t.sum()
        nv = np.sqrt((ub**2).sum(0)); t = np.maximum(nv-1/beta,0); sc = np.where(nv>0, t/np.where(nv>0,nv,1), 0); return ub*sc, t.sum()
    def getg(U, DU, W_):
        Au = A@U; g = At@Au - Atb; V = DU - W_
        lam2 = (V**2).sum(); lam4 = (sig*V).sum(); lam3 = ((Au-b)**2).sum(); lam5 = (delta*(Au-b)).sum()
        g2 = Dtop(V, dims); return Au, g, g2, lam2, lam3, lam4, lam5
    DU = Dop(U, dims); W_, lam1 = shrink(DU)
    Au, g, g2, lam2, lam3, lam4, lam5 = getg(U, DU, W_)
    F = lambda: lam1 + beta/2*lam2 + mu/2*lam3 - lam4 - lam5
    f = F(); d = g2 + mu/beta*g + DtsAtd
    rcdU = U.copy()
    Q, C = 1.0, f; outer = total = 0; uup = None
    nbt = nrs = 0
    while outer < o['maxcnt'] and total < o['maxit']:
        fst = True
        while total < o['maxit']:
            if fst:
                Dd = Dop(d, dims); Ad = A@d
                tau = abs((d@d)/((Dd**2).sum() + mu/beta*(Ad@Ad)))
            else:
                ss = uup@uup; sy = uup@((g2-g2p) + mu/beta*(g-gp)); tau = abs(ss/sy)
            Up, gp, g2p, Aup, DUp = U, g, g2, Au, DU
            U = U - tau*d
            if o['nonneg']: U = np.maximum(U, 0)
            DU = Dop(U, dims)
            Au, g, g2, lam2, lam3, lam4, lam5 = getg(U, DU, W_); f = F()
            alpha = 1.0; dU = U - Up; carm = (d@d)*tau*o['c']*beta
            if abs(f) > abs(C - alpha*carm):
                dg, dg2, dAu, dDU = g-gp, g2-g2p, Au-Aup, DU-DUp; cnt = 0
                while abs(f) > abs(C - alpha*carm):
                    if cnt == 5:
                        gam *= o['rate_gam']
                        Dd = Dop(d, dims); Ad = A@d
                        tau = abs((d@d)/((Dd**2).sum() + mu/beta*(Ad@Ad)))
                        U = np.maximum(Up - tau*d, 0) if o['nonneg'] else Up - tau*d
                        DU = Dop(U, dims); Au, g, g2, lam2, lam3, lam4, lam5 = getg(U, DU, W_); f = F(); nrs += 1
                        break
                    alpha *= o['gamma']
                    g, g2, U, Au, DU = gp+alpha*dg, g2p+alpha*dg2, Up+alpha*dU, Aup+alpha*dAu, DUp+alpha*dDU
                    V = DU - W_; lam2 = (V**2).sum(); lam4 = (sig*V).sum(); lam3 = ((Au-b)**2).sum(); lam5 = (delta*(Au-b)).sum(); f = F()
                    cnt += 1; nbt += 1
            f -= lam1 + beta/2*lam2 - lam4
            W_, lam1 = shrink(DU); V = DU - W_; lam2 = (V**2).sum(); lam4 = (sig*V).sum(); g2 = Dtop(V, dims)
            f += lam1 + beta/2*lam2 - lam4
            Qp = Q; Q = gam*Qp + 1; C = (gam*Qp*C + f)/Q
            uup = U - Up; d = g2 + mu/beta*g + DtsAtd; total += 1
            nrmup = np.linalg.norm(Up); relchg = np.linalg.norm(uup)/nrmup
            if relchg < o['tol_inn'] and not fst: break
            fst = False
        outer += 1
        relout = np.linalg.norm(U - rcdU)/nrmup; rcdU = U.copy()
        if relout < o['tol']: break
        f += lam4 + lam5; V = DU - W_; sig = sig - beta*V; lam4 = (sig*V).sum(); Aub = Au - b; delta = delta - mu*Aub; lam5 = delta@Aub; f -= lam4 + lam5
        beta0 = beta; beta = min(beta*o['rate_cnt'], o['beta']); mu = min(mu*o['rate_cnt'], o['mu'])
        f = F(); DtsAtd = beta0/beta*d; d = g2 + mu/beta*g + DtsAtd; gam = o['gam']; Q = 1; C = f
    return U/scl, dict(total=total, outer=outer, bt=nbt, rs=nrs)

