"""The CPU oracle against the reference: golden vectors and (where the
reference was built on this machine) live runs of oracle/_ref."""
import numpy as np
import pytest

from conftest import golden_manifest, load_golden

MANIFEST = golden_manifest()
SINGLE = sorted(k for k, v in MANIFEST.items() if "ntask" not in v)
LISTS = sorted(k for k, v in MANIFEST.items() if "ntask" in v)


def _kernel(O, meta, g):
    hi = g["hi"] if g["hi"].size > 1 else None
    return O.make_kernel(meta["type"], **meta["params"], **({"hi": hi, "hj": hi} if hi is not None else {}))


@pytest.mark.parametrize("name", SINGLE)
def test_oracle_matches_reference_golden(oracle_mod, name):
    O, meta, g = oracle_mod, MANIFEST[name], load_golden(name)
    ker = _kernel(O, meta, g)
    u = g["u0"].copy()
    rc = O.dgsks(ker, u, g["umap"], g["X"], g["X2"], g["amap"], g["X"], g["X2"], g["bmap"], g["w"], g["wmap"])
    assert rc == 0
    # the reference's own acceptance test uses 1e-13 normwise (test/test_dgsks.c:41,75)
    assert O.errors(u, g["u_ref"])["normwise"] <= 1e-13
    # The reference's fused dgsks is singular for Laplace at coincident points: its
    # assembled d2 is rounding noise instead of 0 and K overflows, while dgsks_ref
    # cancels exactly and applies its clamp (frame/dgsks_ref.c:343-345).
    singular = meta["type"] == O.KS_LAPLACE and np.intersect1d(g["amap"], g["bmap"]).size > 0
    if not singular:
        assert O.errors(u, g["u_dgsks"])["normwise"] <= 1e-12
    # untouched u entries stay bit-identical
    touched = np.zeros(u.size, bool); touched[g["umap"]] = True
    assert np.array_equal(u[~touched], g["u0"][~touched])
    # Laplace overwrites the descriptor exactly as the reference does
    assert ker.powe == float(g["powe_after"]) and ker.scal == float(g["scal_after"])


@pytest.mark.parametrize("name", ["gauss_general", "laplace_k37", "poly3_general", "gauss_k300", "varbw_general"])
def test_fused_port_matches_oracle(oracle_mod, name):
    O, meta, g = oracle_mod, MANIFEST[name], load_golden(name)
    u = g["u0"].copy()
    O.dgsks(_kernel(O, meta, g), u, g["umap"], g["X"], g["X2"], g["amap"], g["X"], g["X2"], g["bmap"], g["w"], g["wmap"], impl="fused")
    assert O.errors(u, g["u_ref"])["normwise"] <= 1e-13


@pytest.mark.parametrize("name", ["gauss_general", "tanh_general", "laplace_general"])
def test_sampled_rows_match_full(oracle_mod, name):
    O, meta, g = oracle_mod, MANIFEST[name], load_golden(name)
    rows = np.arange(0, meta["m"], 7, dtype=np.int32)
    s, a = O.rows(_kernel(O, meta, g), rows, g["X"], g["X2"], g["amap"], g["X"], g["X2"], g["bmap"], g["w"], g["wmap"])
    ref = g["u_ref"][g["umap"][rows]] - g["u0"][g["umap"][rows]]
    assert np.all(np.abs(s - ref) <= 1e-12 * np.maximum(a, 1e-300) + 1e-15)
    assert np.all(a >= np.abs(s) * (1 - 1e-12))


@pytest.mark.parametrize("name", LISTS)
def test_list_oracle_matches_reference(oracle_mod, name):
    O, meta, g = oracle_mod, MANIFEST[name], load_golden(name)
    u = g["u0"].copy()
    ker = O.make_kernel(meta["type"], **meta["params"])
    rc = O.dgsks_list(ker, u, g["a_off"], g["a_idx"], g["a_idx"], g["b_off"], g["b_idx"], g["b_idx"],
                      g["X"], g["X2"], g["X"], g["X2"], g["w"])
    assert rc == 0
    assert O.errors(u, g["u_ref"])["normwise"] <= 1e-13
    # omp_dgsks_list (per-thread u_local + merge) vs the per-task dgsks_ref loop:
    # the reference's own per-entry check is 1e-10 (test/test_dgsks_list.cpp:241-247)
    assert O.errors(g["u_list"], g["u_ref"])["normwise"] <= 1e-12
    assert O.errors(u, g["u_list"])["normwise"] <= 1e-12
    # the multi-threaded list baseline (per-thread copies of u, then a merge)
    u2 = g["u0"].copy()
    assert O.dgsks_list(O.make_kernel(meta["type"], **meta["params"]), u2, g["a_off"], g["a_idx"], g["a_idx"],
                        g["b_off"], g["b_idx"], g["b_idx"], g["X"], g["X2"], g["X"], g["X2"], g["w"],
                        impl="omp") == 0
    assert O.errors(u2, g["u_list"])["normwise"] <= 1e-12


def test_illegal_type_reports(oracle_mod):
    O = oracle_mod
    g = load_golden("gauss_m1n1")
    ker = O.make_kernel(9)
    u = g["u0"].copy()
    assert O.dgsks(ker, u, g["umap"], g["X"], g["X2"], g["amap"], g["X"], g["X2"], g["bmap"], g["w"], g["wmap"]) == -1


@pytest.mark.parametrize("ktype", range(8))
def test_live_against_reference(oracle_mod, ktype):
    """Fresh seeded inputs through oracle/_ref (only where it was built)."""
    O = oracle_mod
    if not O.reference_available():
        pytest.skip("reference library not built on this machine")
    rng = np.random.default_rng(100 + ktype)
    N, k, m, n = 400, 11, 170, 190
    X = np.floor(rng.random((N, k)) * 100) / 1000.0
    X2 = O.norms(X)
    w = rng.standard_normal(N)
    amap = rng.choice(N, m, replace=False).astype(np.int32)
    bmap = rng.choice(N, n, replace=False).astype(np.int32)
    umap = rng.permutation(N)[:m].astype(np.int32)
    wmap = rng.permutation(N)[:n].astype(np.int32)
    s = 1.0 + 0.5 / (1.0 + np.exp(-X2)); hi = -1.0 / (2 * s * s)
    params = {0: dict(scal=-0.5), 1: dict(powe=3.0, scal=0.1, cons=0.1), 2: {}, 3: dict(hi=hi, hj=hi),
              4: dict(scal=0.1, cons=0.1), 5: {}, 6: dict(cons=1.0), 7: {}}[ktype]
    out = {}
    for impl in ("oracle", "reference"):
        u = np.zeros(N)
        O.dgsks(O.make_kernel(ktype, **params), u, umap, X, X2, amap, X, X2, bmap, w, wmap, impl=impl)
        out[impl] = u
    assert O.errors(out["oracle"], out["reference"])["normwise"] <= 1e-13
