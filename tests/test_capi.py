"""The C-ABI driven from a C program (tests/c/capi_driver.c), built with gcc
against include/ncg.h and linked to libncg.so, as a GObject wrapper would use
it.  The build and a GPU-free call run on CPU; the full sequence (reset,
add_obs, prepare, eval_m2lnp, sample, prepare_interp, per-point eval, get_Ki)
runs on the GPU and is checked against the golden fixtures: -2 ln p and the
sampled points <= 1e-10 relative, kernel indices bit-exact, weights <= 1e-10
relative to the largest weight."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden, rel_err


@pytest.fixture(scope="module")
def driver(ng, tmp_path_factory):
    from numcosmo_gb300 import _lib

    libdir = os.path.dirname(_lib.lib_path())
    exe = str(tmp_path_factory.mktemp("capi") / "capi_driver")
    subprocess.run(["gcc", "-O2", "-std=c11", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c", "capi_driver.c"), "-o", exe, "-L", libdir, "-lncg",
                    f"-Wl,-rpath,{libdir}"], check=True)
    return exe


def test_c_program_links_and_calls(driver):
    out = subprocess.run([driver, "--version"], check=True, capture_output=True, text=True).stdout
    assert "sm_103a" in out
    assert "the sample is too small" in out


@pytest.mark.gpu
def test_c_program_full_sequence(gpu, driver, tmp_path):
    """Gaussian VKDE d=12, N=512 (the golden weight-fit case): the C program's
    results against the golden fixture and the Python binding on the same draws."""
    ng = gpu
    g = golden("vkde_gauss_interp_d12_n512")
    d, n, m, ns = 12, g["centres"].shape[0], g["points"].shape[0], 256
    u, z, _ = ng.RNG(11).sample_stream(ng.StatsDistKernelGauss(d), ns)
    for name, a in (("centres", g["centres"]), ("points", g["points"]), ("u", u), ("z", z), ("target", g["target"])):
        np.ascontiguousarray(a, dtype=np.float64).tofile(tmp_path / f"{name}.f64")
    r = subprocess.run([driver, str(tmp_path), "1", "0", str(d), "3.0", str(n), str(m), str(ns)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr

    # before the fit: equal weights, as prepare leaves them
    sd = ng.StatsDistVKDE(ng.StatsDistKernelGauss(d), ng.StatsDistCV.NONE)
    sd.set_sample(g["centres"])
    sd.prepare()
    assert rel_err(np.fromfile(tmp_path / "m2lnp.f64"), sd.eval_m2lnp(g["points"])) < 1e-10
    xw, iw = sd.sample(u, z)
    x = np.fromfile(tmp_path / "x.f64").reshape(ns, d)
    assert np.array_equal(np.fromfile(tmp_path / "idx.i32", dtype=np.int32), iw)
    assert np.max(np.abs(x - xw)) <= 1e-10 * max(1.0, np.max(np.abs(xw)))

    # after the fit: the golden weights and -2 ln p
    w = np.fromfile(tmp_path / "weights.f64")
    assert np.max(np.abs(w - g["weights"])) <= 1e-10 * np.max(g["weights"])
    assert rel_err(np.fromfile(tmp_path / "m2lnp_fit.f64"), g["m2lnp"]) < 1e-10
    sd.prepare_interp(g["target"])
    y0, cov0, n0, w0 = sd.get_Ki(0)
    Ki = np.fromfile(tmp_path / "Ki.f64")
    assert np.array_equal(Ki[:d], y0)
    assert rel_err(Ki[d:d + d * d], cov0.ravel(), floor=1e-3) < 1e-12
    assert Ki[-2] == pytest.approx(n0, rel=1e-12) and Ki[-1] == pytest.approx(w0, rel=1e-10)
