"""The More-Thuente line search (superdca_gb300/csrc/linesearch.h), the
state machine every engine form runs (on the host for the tensor-core and
plain forms, inside k_dual_linesearch for the dual form), on one-dimensional
functions with known shapes: it must stop at a point that satisfies the
strong Wolfe conditions SuperDCA's LbfgsSolver asks for (ftol 1e-4, gtol
1e-2) within its 20 evaluations, from starting steps spread over six
orders of magnitude.  Compiled with the host compiler: no GPU."""
import json
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r"""
#include <cmath>
#include <cstdio>
#include "linesearch.h"

// value and derivative of each test function at a
static void fn(int k, double a, double *f, double *g)
{
    switch (k) {
    case 0: {  // -a / (a^2 + 2): minimum at sqrt(2)
        const double d = a * a + 2.0;
        *f = -a / d;
        *g = (a * a - 2.0) / (d * d);
        break;
    }
    case 1: {  // (a + b)^5 - 2 (a + b)^4, b = 0.004: minimum at 1.6 - b
        const double t = a + 0.004;
        *f = std::pow(t, 5) - 2.0 * std::pow(t, 4);
        *g = 5.0 * std::pow(t, 4) - 8.0 * std::pow(t, 3);
        break;
    }
    case 2: {  // 0.5 (a - 3)^2
        *f = 0.5 * (a - 3.0) * (a - 3.0);
        *g = a - 3.0;
        break;
    }
    case 3: {  // log(1 + exp(-4 a)) + 0.01 a^2: a logistic term plus an L2 term
        const double e = std::exp(-4.0 * a);
        *f = std::log1p(e) + 0.01 * a * a;
        *g = -4.0 * e / (1.0 + e) + 0.02 * a;
        break;
    }
    default: {  // a dip that flattens out, then a shallow L2 bowl: -a^2 / (1 + a^2) - 0.01 a + 1e-4 a^2
        const double d = 1.0 + a * a;
        *f = -a * a / d - 0.01 * a + 1e-4 * a * a;
        *g = -2.0 * a / (d * d) - 0.01 + 2e-4 * a;
        break;
    }
    }
}

int main()
{
    const double starts[] = {1e-3, 1e-2, 1e-1, 1.0, 10.0, 1e3};
    std::printf("[");
    bool first = true;
    for (int k = 0; k < 5; ++k)
        for (double a0 : starts) {
            double f0, g0;
            fn(k, 0.0, &f0, &g0);
            sdca::MoreThuente mt;
            int evals = 0;
            double f = f0, g = g0, stp = 0.0;
            if (mt.start(f0, g0, a0) == sdca::MoreThuente::NEED_EVAL) {
                for (;;) {
                    stp = mt.stp;
                    fn(k, stp, &f, &g);
                    ++evals;
                    if (mt.feed(f, g) == sdca::MoreThuente::DONE || evals > 64) break;
                }
            }
            std::printf("%s{\"fn\": %d, \"a0\": %.17g, \"stp\": %.17g, \"f\": %.17g, \"g\": %.17g, \"f0\": %.17g, "
                        "\"g0\": %.17g, \"evals\": %d, \"info\": %d}",
                        first ? "" : ", ", k, a0, stp, f, g, f0, g0, evals, mt.info);
            first = false;
        }
    std::printf("]\n");
    return 0;
}
"""


@pytest.fixture(scope="module")
def runs(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    d = tmp_path_factory.mktemp("ls")
    src, exe = d / "ls.cpp", d / "ls"
    src.write_text(SRC)
    inc = os.path.join(ROOT, "superdca_gb300", "csrc")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I" + inc, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return json.loads(out)


def test_every_search_ends_at_a_strong_wolfe_point(runs):
    assert len(runs) == 30
    for r in runs:
        assert r["evals"] <= 20, r
        assert r["info"] == 1, r                                           # both tests met
        assert r["f"] <= r["f0"] + 1e-4 * r["stp"] * r["g0"] + 1e-15, r    # sufficient decrease
        assert abs(r["g"]) <= 1e-2 * abs(r["g0"]) + 1e-15, r               # curvature


def test_searches_from_small_steps_extrapolate(runs):
    """Starting 1000x below the minimiser, the search grows the step (by up
    to 4x the last extrapolation per trial) instead of stopping early."""
    for r in runs:
        if r["a0"] == 1e-3:
            assert r["stp"] > 0.1, r
