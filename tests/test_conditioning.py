"""Why the FP32-LU form is not the default: the Newton systems of the c2 workload are too
badly conditioned for FP32 factorisation with FP64 refinement.  Systems from the oracle's
restatement of the system build (first iteration, 100x the initial step), row- and
column-equilibrated by powers of two: the condition numbers exceed 1e8, and FP32 LU with
up to 3 FP64-residual refinements (the library's mixed form, in numpy) reaches the form's
stop criterion for few of them."""
import numpy as np

import workloads


def _lu32(A):
    L = A.astype(np.float32).copy()
    for k in range(A.shape[0]):
        L[k + 1:, k] /= L[k, k]
        L[k + 1:, k + 1:] -= np.outer(L[k + 1:, k], L[k, k + 1:])
    return L


def _solve32(L, r):
    d = r.astype(np.float32).copy()
    n = L.shape[0]
    for k in range(n):
        d[k + 1:] -= L[k + 1:, k] * d[k]
    for k in range(n - 1, -1, -1):
        d[k] /= L[k, k]
        d[:k] -= L[:k, k] * d[k]
    return d.astype(np.float64)


def test_c2_newton_systems_defeat_fp32_refinement(port):
    w = workloads.make("c2", P=24, seed=3)
    kappas, settled = [], 0
    for i in range(24):
        A, b = port.newton_system(86, w["Y"][:, i], w["T"][i], w["rho"][i], w["dt"][i] * 100, eos="helmholtz")
        r = 2.0 ** -np.floor(np.log2(np.abs(A).max(1)))
        As = A * r[:, None]
        c = 2.0 ** -np.floor(np.log2(np.abs(As).max(0)))
        kappas.append(np.linalg.cond(As * c[None, :]))
        L = _lu32(As)
        x, res = np.zeros(87), b.copy()
        state = np.concatenate([[w["T"][i]], np.abs(w["Y"][:, i])])
        for _ in range(4):  # the first solve and up to 3 refinements
            d = _solve32(L, res * r)
            x += d
            if np.all(np.isfinite(x)) and np.all(np.abs(d) <= 2.0 ** -50 * (np.abs(x) + state)):
                settled += 1
                break
            res = b - A @ x
    assert np.median(kappas) > 1e8, np.median(kappas)
    assert settled < 12, settled
