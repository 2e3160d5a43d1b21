"""Stand-in electron-positron Helmholtz free-energy table (541 x 201 grid).

The Helmholtz EOS interpolates a table of the electron free energy f(den, T) and its
derivatives (den = rho * Ye).  The table the reference reads at static-initialisation
time (include/nnet/parameterization/eos/helmholtz.cpp:89-172) is not shipped with it,
so this module generates a thermodynamically consistent stand-in on the same grid
(helmholtz.hpp:77-88: log10 den in [-12, 15] with 541 points, log10 T in [3, 13] with
201 points) and in the same quantities:

  f, fd, ft, fdd, ftt, fdt, fddt, fdtt, fddtt      free energy and derivatives
  dpdf, dpdfd, dpdft, dpdfdt                       dP/dden and derivatives
  ef, efd, eft, efdt                               electron chemical potential / kT
  xf, xfd, xft, xfdt                               electron number density

Model (per gram of `den`; all derivatives analytic):
  * a Maxwell-Boltzmann ideal electron gas, f_th = NA k T (ln(ne lambda^3 / 2) - 1),
    ne = NA den, lambda = h / sqrt(2 pi me k T);
  * plus the T = 0 kinetic energy of a relativistic degenerate electron gas,
    f_deg = eps_k(ne) / den, with x = p_F / (me c) and the exact Chandrasekhar
    pressure; small x uses the series of eps_k to avoid cancellation.
Pair production and finite-temperature degeneracy corrections are left out, so the
electron heat capacity is 1.5 NA k per gram of den.  The table is a smooth, positive,
derivative-consistent surrogate; GPU kernels and the CPU oracle read the same bytes.

Binary layout written by `generate`: 21 float64 arrays in the order above, each
[IMAX][JMAX] (row i = density index, column j = temperature index), 18,264,780 bytes.
`write_reference_text` writes the reference's text layout (helmholtz.cpp:100-137).
"""
import os
import sys

import numpy as np

IMAX, JMAX = 541, 201
TLO, THI, DLO, DHI = 3.0, 13.0, -12.0, 15.0

# physical constants of the Helmholtz EOS (helmholtz.hpp:93-105)
H = 6.6260689633e-27
HBAR = 0.5 * H / np.pi
AVO = 6.0221417930e23
CLIGHT = 2.99792458e10
KERG = 1.380650424e-16
ME = 9.1093821545e-28

NAMES = ["f", "fd", "ft", "fdd", "ftt", "fdt", "fddt", "fdtt", "fddtt",
         "dpdf", "dpdfd", "dpdft", "dpdfdt",
         "ef", "efd", "eft", "efdt",
         "xf", "xfd", "xft", "xfdt"]


def _grid():
    d = 10.0 ** (DLO + np.arange(IMAX) * ((DHI - DLO) / (IMAX - 1)))
    t = 10.0 ** (TLO + np.arange(JMAX) * ((THI - TLO) / (JMAX - 1)))
    return np.meshgrid(d, t, indexing="ij")


def _degenerate(den):
    """T = 0 electron gas: kinetic energy density, pressure, dP/dden, d2P/dden2, mu."""
    lamc = HBAR / (ME * CLIGHT)
    mc2 = ME * CLIGHT * CLIGHT
    ne = AVO * den
    x = lamc * np.cbrt(3.0 * np.pi ** 2 * ne)
    sq = np.sqrt(1.0 + x * x)
    # eps_k * lamc^3 / (mc2) = (1/pi^2) [ g(x)/8 - x^3/3 ],  g = x(2x^2+1)sqrt(1+x^2) - asinh(x)
    exact = (x * (2 * x * x + 1) * sq - np.arcsinh(x)) / 8.0 - x ** 3 / 3.0
    x2 = x * x
    series = x ** 5 * (1.0 / 10 + x2 * (-1.0 / 56 + x2 * (1.0 / 144 + x2 * (-5.0 / 1408 + x2 * (7.0 / 3328)))))
    eps = np.where(x < 0.1, series, exact) * mc2 / (np.pi ** 2 * lamc ** 3)
    mu = mc2 * x2 / (sq + 1.0)                       # kinetic chemical potential
    p = ne * mu - eps                                # pressure
    dp = AVO * mc2 * x2 / (3.0 * sq)                 # dP/dden
    ddp = AVO * mc2 * x2 * (2.0 + x2) / (9.0 * den * sq ** 3)
    dmu = mc2 * x2 / (3.0 * den * sq)                # dmu/dden
    return eps, p, dp, ddp, mu, dmu


def tables():
    return evaluate(*_grid())


def evaluate(d, t):
    """All 21 quantities of the model at density d (= rho Ye) and temperature t."""
    d, t = np.asarray(d, dtype=np.float64), np.asarray(t, dtype=np.float64)
    nak = AVO * KERG
    lam3 = (H * H / (2.0 * np.pi * ME * KERG * t)) ** 1.5
    lnpsi = np.log(AVO * d * lam3 / 2.0)
    eps, p, dp, ddp, mu, dmu = _degenerate(d)

    out = {}
    out["f"] = nak * t * (lnpsi - 1.0) + eps / d
    out["fd"] = nak * t / d + p / (d * d)
    out["ft"] = nak * (lnpsi - 2.5)
    out["fdd"] = -nak * t / (d * d) + dp / (d * d) - 2.0 * p / d ** 3
    out["ftt"] = -1.5 * nak / t
    out["fdt"] = nak / d
    out["fddt"] = -nak / (d * d)
    out["fdtt"] = np.zeros_like(d)
    out["fddtt"] = np.zeros_like(d)

    out["dpdf"] = nak * t + dp
    out["dpdfd"] = ddp
    out["dpdft"] = np.full_like(d, nak)
    out["dpdfdt"] = np.zeros_like(d)

    kt = KERG * t
    out["ef"] = lnpsi + mu / kt
    out["efd"] = 1.0 / d + dmu / kt
    out["eft"] = -1.5 / t - mu / (kt * t)
    out["efdt"] = -dmu / (kt * t)

    out["xf"] = AVO * d
    out["xfd"] = np.full_like(d, AVO)
    out["xft"] = np.zeros_like(d)
    out["xfdt"] = np.zeros_like(d)
    return out


def generate(path):
    """Write the binary table (21 x IMAX x JMAX float64, little endian)."""
    tab = tables()
    arr = np.stack([tab[n] for n in NAMES]).astype("<f8")
    assert np.all(np.isfinite(arr))
    tmp = path + ".tmp"
    arr.tofile(tmp)
    os.replace(tmp, path)
    return path


def write_reference_text(path, wrap_str=True):
    """Write the table in the reference's text layout (helmholtz.cpp:100-137)."""
    tab = tables()
    with open(path, "w") as fh:
        if wrap_str:
            fh.write("STR(\n")
        blocks = [NAMES[0:9], NAMES[9:13], NAMES[13:17], NAMES[17:21]]
        for names in blocks:
            # rows ordered j-major then i, each row holding the block's quantities
            cols = np.stack([tab[n].T.reshape(-1) for n in names], axis=1)
            np.savetxt(fh, cols, fmt="%.17e")
        if wrap_str:
            fh.write(")\n")
    return path


if __name__ == "__main__":
    generate(sys.argv[1] if len(sys.argv) > 1 else "helm_table.bin")
