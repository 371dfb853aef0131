"""The algorithmic work per bin that the roofline figure in bench.py uses.

oracle/opcount.cpp instantiates the oracle's templated per-bin arithmetic (the bodies
of the reference's collect_rt_cpu! and collect_cb_cpu! bin loops, src/cpu.jl:13-26,
85-126, 132-156) with an operation-counting scalar type. This test builds and runs it
and checks that bench.py's flop constants are the counted ones, so the roofline's
"achieved" figure is the reference algorithm's operation count, not an estimate.
"""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def counts():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    out = subprocess.run([os.path.join(ROOT, "oracle", "_build", "opcount"), "200"], check=True,
                         capture_output=True, text=True).stdout
    return json.loads(out)


def test_bench_flops_are_the_counted_ones(counts):
    sys.path.insert(0, ROOT)
    import bench

    mie = counts["mie"]
    assert bench.FLOPS_RT_MIE == pytest.approx(mie["rt_bin"]["flops"], rel=2e-3)
    assert bench.FLOPS_CBN_MIE == pytest.approx(mie["cb_reciprocal_bin"]["flops"], rel=2e-3)
    assert bench.FLOPS_CB1_MIE == pytest.approx(mie["cb_single_bin"]["flops"], rel=2e-3)


def test_counts_have_the_expected_structure(counts):
    for kind in ("rayleigh", "mie"):
        c = counts[kind]
        # an RT bin calls update_I once; a reciprocal-path CB bin calls update_E twice
        # and I_from_E three times, so it costs at least twice an RT bin
        assert c["cb_reciprocal_bin"]["flops"] > 2 * c["rt_bin"]["flops"]
        assert c["cb_reciprocal_bin"]["sincos"] == pytest.approx(2.0)  # exp(i dPhi)
        assert c["cb_reciprocal_bin"]["exp"] == pytest.approx(2.0)
        assert 0.5 < c["rt_bin"]["exp"] <= 1.0  # tau0 cuts some grazing bins
    # the Mie lookups add one arccos per phase or amplitude matrix
    assert counts["mie"]["rt_bin"]["acos"] == pytest.approx(1.0)
    assert counts["mie"]["cb_reciprocal_bin"]["acos"] == pytest.approx(2.0)
    assert counts["rayleigh"]["rt_bin"]["acos"] == 0.0
