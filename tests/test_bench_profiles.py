"""bench.py's roofline line reads the DRAM traffic of its dominant kernel from
the committed ncu summaries: every kernel of the step has one, with a number."""
import importlib.util
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_each_step_kernel_has_a_traffic_figure():
    b = _bench()
    for name, _kt, _p, _f in b.KERNELS:
        for form in ("split_tiles", "fp64_tiles"):
            prof = f"{form}_{name}_general_stride"
            if form == "fp64_tiles" and name != "gaussian":
                continue                      # the FP64 form is profiled on its Gaussian only
            v = b.read_traffic(prof)
            assert v is not None and v > 0, prof


def test_profiles_name_their_commands():
    pdir = os.path.join(ROOT, "profiles")
    names = sorted(f for f in os.listdir(pdir) if f.endswith(".md"))
    assert names
    for f in names:
        text = open(os.path.join(pdir, f)).read()
        assert "ncu " in text and "--clock-control none" in text, f
