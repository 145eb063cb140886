"""The C++ drop-in ScaFES::Problem without a GPU: problem classes written
against the ScaFES callback interface compile against the drop-in headers,
and the stencil extraction maps their updates to the expected device form
(or refuses them with a message).  Where the reference checkout exists, the
reference's own system-test classes are compiled unchanged and checked the
same way."""
from __future__ import annotations

import subprocess
from pathlib import Path

import pytest

from dropin.build import HERE, REFERENCE, compile_cpp


@pytest.fixture(scope="module")
def run_problem(native, tmp_path_factory):
    return compile_cpp(HERE / "run_problem.cpp", tmp_path_factory.mktemp("dropin") / "run_problem")


def form(exe, *args):
    out = subprocess.run([str(exe), *args], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    return out.stdout


@pytest.mark.parametrize("name,expect", [
    ("heat_lin", ["c0=0.02 ", "cp=(0.163333,0.163333,0.163333)", "source=static", "border=dirichlet"]),
    ("pennes_lin", ["c0=0.0166667", "source=affine", "border=dirichlet"]),
    ("mirror_pow2", ["c0=0.285714", "source=none", "border=mirror"]),
    ("heat_neumann", ["c0=0.02 ", "source=static", "border=table"]),
    ("heat_cauchy", ["c0=0.02 ", "source=static", "border=table"]),
    ("pennes_radiation", ["source=affine", "border=table", "G=quartic-in-time", "u^4"]),
])
def test_extracted_form(run_problem, name, expect):
    s = form(run_problem, name, "/dev/null", "--extract-only", "--nNodes=8x8x8", "--nTimesteps=300", "--endtime=1")
    for e in expect:
        assert e in s, s


REF_SYS = REFERENCE / "tests" / "system"
REF_CASES = [
    (1, ["HeatEqnFDM", "HeatEqnFDM/Dirichlet", "HeatEqnFDM/Dirichlet/TimeLinSpaceLin"], "FORM star7 c0=0.02 ", "border=dirichlet"),
    (2, ["PennesBioheatEqnFDM", "PennesBioheatEqnFDM/Dirichlet", "PennesBioheatEqnFDM/Dirichlet/TimeLinSpaceLin"],
     "source=affine", "border=dirichlet"),
    (3, ["HeatEqnFdmStencilWidthOne"], "c0=0.285714", "border=mirror"),
    (4, ["HeatEqnFDM", "HeatEqnFDM/Neumann", "HeatEqnFDM/Neumann/TimeLinSpaceLin"], "FORM star7 c0=0.02 ",
     "border=table"),
    (6, ["HeatEqnFDM", "HeatEqnFDM/Cauchy", "HeatEqnFDM/Cauchy/TimeLinSpaceLin"], "FORM star7 c0=0.02 ",
     "border=table"),
    (7, ["PennesBioheatEqnFDM", "PennesBioheatEqnFDM/Neumann", "PennesBioheatEqnFDM/Neumann/TimeLinSpaceLin"],
     "source=affine", "border=table"),
    (8, ["PennesBioheatEqnFDM", "PennesBioheatEqnFDM/Radiation",
         "PennesBioheatEqnFDM/Radiation/TimeLinSpaceLin"], "border=table G=quartic-in-time u^4", "source=affine"),
    (5, ["PropagationFromLeftLowerCorner"], "REFUSED", "branches on the value"),
]


@pytest.mark.skipif(not (REF_SYS / "HeatEqnFDM").exists(), reason="reference checkout not present")
@pytest.mark.parametrize("pid,dirs,e1,e2", REF_CASES)
def test_reference_system_test_classes_unchanged(native, tmp_path, pid, dirs, e1, e2):
    extra = [f"-DPROBLEM={pid}"] + sum((["-I", str(REF_SYS / d)] for d in dirs), [])
    exe = compile_cpp(HERE / "extract_reference.cpp", tmp_path / f"xref{pid}", extra)
    s = form(exe, "--nNodes=8x8x8", "--nTimesteps=300", "--endtime=1")
    assert e1 in s and e2 in s, s
