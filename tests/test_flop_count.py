"""The algorithmic FP64 operation counts the benchmark reports are the
oracle's: every float64 add, multiply, division and square root of one RK3
step of the TGV workload, per interior cell-update (n^3 coefficient over
four grid sizes)."""
import importlib.util
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_module", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_tgv_flop_count_matches_the_benchmark_constant():
    from oracle import flop_count
    r = flop_count.per_cell_update(flop_count.TGV)
    assert r["flop"] == pytest.approx(_bench().FP64_FLOP_ALGORITHMIC["tgv"], abs=0.5)
    assert r["div"] == pytest.approx(490.0, abs=0.5) and r["sqrt"] == pytest.approx(46.0, abs=0.5)


def test_viscous_flop_count_matches_the_benchmark_constant():
    from oracle import flop_count
    r = flop_count.per_cell_update(flop_count.VISCOUS_TGV)
    assert r["flop"] == pytest.approx(_bench().FP64_FLOP_ALGORITHMIC["viscous"], abs=0.5)
