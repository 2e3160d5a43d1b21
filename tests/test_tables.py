"""Stand-in Helmholtz table: thermodynamic and derivative consistency of the generator,
and the binary / reference-text writers agree."""
import numpy as np

import gen_helm_table as G


def num_d(q, d, t, h=1e-5):
    return (G.evaluate(d * (1 + h), t)[q] - G.evaluate(d * (1 - h), t)[q]) / (2 * h * d)


def num_t(q, d, t, h=1e-5):
    return (G.evaluate(d, t * (1 + h))[q] - G.evaluate(d, t * (1 - h))[q]) / (2 * h * t)


def test_derivatives_consistent():
    rng = np.random.default_rng(0)
    d = 10 ** rng.uniform(-6, 12, 64)
    t = 10 ** rng.uniform(6, 11, 64)
    v = G.evaluate(d, t)
    pairs = [("fd", num_d("f", d, t)), ("ft", num_t("f", d, t)), ("fdd", num_d("fd", d, t)),
             ("ftt", num_t("ft", d, t)), ("fdt", num_t("fd", d, t)), ("dpdf", num_d("f", d, t) * 0)]
    for name, ref in pairs[:-1]:
        rel = np.abs(v[name] - ref) / np.maximum(np.abs(v[name]), 1e-300)
        assert np.median(rel) < 1e-6 and rel.max() < 1e-3, name
    # pressure P = d^2 df/dd and dP/dd
    P = lambda dd: dd ** 2 * G.evaluate(dd, t)["fd"]
    dP = (P(d * (1 + 1e-5)) - P(d * (1 - 1e-5))) / (2e-5 * d)
    assert np.median(np.abs(dP - v["dpdf"]) / v["dpdf"]) < 1e-6


def test_positive_heat_capacity_and_pressure():
    tab = G.tables()
    assert np.all(tab["ftt"] < 0)           # c_v = -T d2f/dT2 > 0
    assert np.all(tab["dpdf"] > 0) and np.all(tab["fd"] > 0)


def test_text_writer_layout(tmp_path):
    path = G.write_reference_text(str(tmp_path / "helm_table.dat"))
    txt = open(path).read()
    assert txt.startswith("STR(") and txt.rstrip().endswith(")")
    body = np.array(txt[4:txt.rindex(")")].split(), dtype=np.float64)
    assert body.size == 541 * 201 * 21
    tab = G.tables()
    # first row of the f block: (j=0, i=0), quantities f fd ft fdd ftt fdt fddt fdtt fddtt
    assert np.array_equal(body[:9], np.array([tab[n][0, 0] for n in G.NAMES[:9]]))
