"""ctypes front end of the oracle libraries (test infrastructure only).

`Oracle("port")` loads oracle/liboracle.so (the CPU restatement, buildable anywhere);
`Oracle("ref")` loads oracle/_ref/libnnet_ref.so (the reference's own sources, built only
where the reference tree exists).  Both expose the same calls; arrays are numpy float64,
abundances species-major Y[species, particle].
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_D, _P, _I, _L, _S = ctypes.c_double, ctypes.c_void_p, ctypes.c_int, ctypes.c_long, ctypes.c_size_t

STATUS = {0: "OK", 1: "SKIPPED", 2: "LIVELOCK", 3: "MAXITER", 4: "ZERO_DT"}
EOS_FIELDS = ["cv", "dpdT", "p", "cp", "c", "u", "dse", "dpe", "dsp", "cv_gaz", "cp_gaz", "c_gaz", "dudYe"]


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class Oracle:
    def __init__(self, kind="port"):
        if kind == "port":
            path, pre = os.path.join(HERE, "liboracle.so"), "oracle_"
        else:
            path, pre = os.path.join(HERE, "_ref", "libnnet_ref.so"), "ref_"
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.kind = kind
        self.lib = ctypes.CDLL(path)
        g = lambda n: getattr(self.lib, pre + n)
        self._load = g("load_helmholtz")
        self._load.argtypes = [_P]
        self._helm = g("helmholtz")
        self._helm.argtypes = [_D, _D, _D, _D, _P]
        self._rates = g("rates")
        self._rates.argtypes = [_I, _P, _D, _D, _I, _D, _P, _P, _P, _P]
        self._burn = g("burn")
        self._burn.argtypes = [_I, _I, _D, _S, _P, _P, _P, _P, _P, _D, _D, _I, _L, _P, _P, _P, _I]
        self._nr = g("solve_nr")
        self._nr.argtypes = [_I, _I, _D, _P, _D, _P, _P, _D, _D, _P]
        self._nr.restype = _D
        try:
            self._sys = g("newton_system")
            self._sys.argtypes = [_I, _I, _D, _P, _D, _D, _D, _D, _P, _P]
        except AttributeError:
            self._sys = None
        try:
            self._eosb = g("helm_eos_batch")
            self._eosb.argtypes = [_S, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _I]
        except AttributeError:
            self._eosb = None

    def load_helmholtz(self, table):
        table = np.ascontiguousarray(table, dtype=np.float64)
        assert table.size == 21 * 541 * 201
        self._table = table
        self._load(_ptr(table))

    def helmholtz(self, abar_, zbar_, T, rho):
        out = np.zeros(13)
        self._helm(abar_, zbar_, T, rho, _ptr(out))
        return dict(zip(EOS_FIELDS, out))

    def rates(self, net, Y, T, rho, eos="ideal", mu=10.0):
        nreact = {14: 29, 86: 309, 87: 311}[net]
        Y = np.ascontiguousarray(Y, dtype=np.float64)
        BE, r, dr, e = np.zeros(net), np.zeros(nreact), np.zeros(nreact), np.zeros(13)
        self._rates(net, _ptr(Y), T, rho, 0 if eos == "ideal" else 1, mu, _ptr(BE), _ptr(r), _ptr(dr), _ptr(e))
        return BE, r, dr, dict(zip(EOS_FIELDS, e))

    def burn(self, net, Y, T, rho, dt, hydro_dt, eos="ideal", mu=10.0, rho_m1=None, previous_dt=0.0,
             drhodt_mode=0, max_iter=20000, nthreads=0):
        """Burn in place-copies; returns (Y, T, dt, status, substeps, iters)."""
        Y = np.array(Y, dtype=np.float64, order="C", copy=True)
        T = np.array(T, dtype=np.float64, copy=True)
        dt = np.array(dt, dtype=np.float64, copy=True)
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        rho_m1 = None if rho_m1 is None else np.ascontiguousarray(rho_m1, dtype=np.float64)
        P = T.size
        st, sub, it = np.zeros(P, np.int32), np.zeros(P, np.int32), np.zeros(P, np.int32)
        self._burn(net, 0 if eos == "ideal" else 1, mu, P, _ptr(Y), _ptr(T), _ptr(rho), _ptr(rho_m1), _ptr(dt),
                   hydro_dt, previous_dt, drhodt_mode, max_iter, _ptr(st), _ptr(sub), _ptr(it), nthreads)
        return Y, T, dt, st, sub, it

    def solve_nr(self, net, Y, T, rho, dt, eos="ideal", mu=10.0, drho_dt=0.0):
        Y = np.ascontiguousarray(Y, dtype=np.float64)
        Yo, To, d = np.zeros(net), np.zeros(1), np.array([dt], dtype=np.float64)
        ts = self._nr(net, 0 if eos == "ideal" else 1, mu, _ptr(Y), T, _ptr(Yo), _ptr(To), rho, drho_dt, _ptr(d))
        return Yo, float(To[0]), float(d[0]), ts

    def newton_system(self, net, Y, T, rho, dt, eos="ideal", mu=10.0, drho_dt=0.0):
        """(A, b) of the first Newton iteration of a substep from (Y, T) with step dt;
        index 0 is the temperature, 1.. the species."""
        Y = np.ascontiguousarray(Y, dtype=np.float64)
        n = net + 1
        M, b = np.zeros(n * n), np.zeros(n)
        rc = self._sys(net, 0 if eos == "ideal" else 1, mu, _ptr(Y), T, rho, drho_dt, dt, _ptr(M), _ptr(b))
        if rc:
            raise RuntimeError("newton_system failed")
        return M.reshape(n, n).T.copy(), b

    def helm_eos_batch(self, Z, T, rho, Y, nthreads=0):
        Y = np.ascontiguousarray(Y, dtype=np.float64)
        Z = np.ascontiguousarray(Z, dtype=np.float64)
        T = np.ascontiguousarray(T, dtype=np.float64)
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        P = T.size
        u, cv, p, c, dpdT = (np.zeros(P) for _ in range(5))
        self._eosb(P, Y.shape[0], _ptr(Z), _ptr(T), _ptr(rho), _ptr(Y), _ptr(u), _ptr(cv), _ptr(p), _ptr(c),
                   _ptr(dpdT), nthreads)
        return dict(u=u, cv=cv, p=p, c=c, dpdT=dpdT)


def compare_burns(net, Y0, g, o, tol=1e-8):
    """Per-particle comparison of a GPU burn g = (Y, T, dt, status) with the oracle's o (same
    layout) of the same inputs Y0: relative error of T, of every Y_i > 1e-12 and of the released
    energy E = sum_i BE_i (Y_i - Y0_i) (test infrastructure: the checker of bench.py's baseline
    leg).  Returns a dict of summary figures."""
    import workloads
    Yg, Tg, _, sg = g[:4]
    Yo, To, _, so = o[:4]
    BE = workloads.binding_energies(net)[: Yg.shape[0], None]
    A = np.asarray(workloads.mass_numbers(net), dtype=np.float64)[: Yg.shape[0], None]
    Eg, Eo = (BE * (Yg - Y0)).sum(0), (BE * (Yo - Y0)).sum(0)
    with np.errstate(divide="ignore", invalid="ignore"):
        relT = np.abs(Tg - To) / np.abs(To)
        big = Yo > 1e-12
        relY = np.where(big, np.abs(Yg - Yo) / np.where(big, Yo, 1), 0).max(0)
        relE = np.where(np.abs(Eo) > 0, np.abs(Eg - Eo) / np.abs(Eo), np.abs(Eg - Eo))
    same = sg == so
    tiny_E = np.abs(Eo) < 1e-30 * np.abs(BE).max()
    ok = same & (relT <= tol) & (relY <= tol) & ((relE <= tol) | tiny_E)
    flip = same & ~ok
    dX = (np.abs(Yg - Yo) * A).max(0)
    drift_g, drift_o = (A * Yg).sum(0) - 1, (A * Yo).sum(0) - 1
    mx = lambda a, m: float(a[m].max()) if m.any() else 0.0
    return {"particles": int(sg.size), "within_tol": float(ok.mean()), "tol": tol,
            "status_agree": float(same.mean()), "max_rel_T_within": mx(relT, ok), "max_rel_Y_within": mx(relY, ok),
            "max_rel_E_within": mx(relE, ok), "flipped": int(flip.sum()), "flipped_max_rel_T": mx(relT, flip),
            "flipped_max_abs_dX": mx(dX, flip), "flipped_max_rel_Y": mx(relY, flip),
            "sum_x_drift_max_gpu": float(np.abs(drift_g).max()) if sg.size else 0.0,
            "sum_x_drift_max_oracle": float(np.abs(drift_o).max()) if sg.size else 0.0,
            "sum_x_drift_max_diff": float(np.abs(drift_g - drift_o).max()) if sg.size else 0.0}
