"""C-ABI checks that need no GPU: the library loads, exports every symbol that
include/ncg.h declares, reports status strings, the ctypes mirrors of the public
structs match the header's layout, and its host RNG matches the published
MT19937 known answers and restores a saved state."""
import ctypes as C
import os
import re

import numpy as np
import pytest
import scipy.stats

from conftest import ROOT


def _declared_symbols():
    txt = open(os.path.join(ROOT, "include", "ncg.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = set(re.findall(r"\b(ncg_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


def test_library_exports_every_declared_symbol(ng):
    from numcosmo_gb300 import _lib

    L = _lib.load()
    declared = _declared_symbols()
    assert len(declared) > 40
    missing = [s for s in declared if not hasattr(L, s)]
    assert not missing, missing
    # the ctypes binding covers the whole header
    assert set(declared) <= set(_lib.exported_symbols()), set(declared) - set(_lib.exported_symbols())


def test_version_and_status_strings(ng):
    from numcosmo_gb300 import _lib

    L = _lib.load()
    assert b"sm_103a" in L.ncg_version()
    for code in range(13):
        assert L.ncg_status_string(code)
    assert L.ncg_status_string(2) == b"the sample is too small"


def test_library_is_in_tree_and_sm103a(ng):
    from numcosmo_gb300 import _lib

    path = _lib.lib_path()
    assert path.startswith(os.path.join(ROOT, "numcosmo_gb300"))
    blob = open(path, "rb").read()
    assert b"sm_103a" in blob or b"sm_103" in blob


def test_rng_mt19937_known_answers(ng):
    r = ng.RNG(5489)
    first = [r.get_u32() for _ in range(3)]
    assert first == [3499211612, 581869302, 3890346734]
    for _ in range(9996):
        r.get_u32()
    assert r.get_u32() == 4123659995      # 10000th output of the default seed
    bg = np.random.MT19937(0)
    bg._legacy_seeding(20260721)
    r = ng.RNG(20260721)
    assert [r.get_u32() for _ in range(1000)] == list(bg.random_raw(1000))


def test_rng_transforms_distribution(ng):
    r = ng.RNG(123)
    u = np.array([r.uniform() for _ in range(20000)])
    g = np.array([r.ugaussian() for _ in range(20000)])
    c = np.array([r.chisq(3.0) for _ in range(20000)])
    c7 = np.array([r.chisq(0.7) for _ in range(20000)])
    assert scipy.stats.kstest(u, "uniform").pvalue > 1e-3
    assert scipy.stats.kstest(g, "norm").pvalue > 1e-3
    assert scipy.stats.kstest(c, scipy.stats.chi2(3.0).cdf).pvalue > 1e-3
    assert scipy.stats.kstest(c7, scipy.stats.chi2(0.7).cdf).pvalue > 1e-3


def test_rng_sample_stream_order(ng):
    """One sample call consumes u, then dim gaussians, then chi^2 (Student-t)."""
    k = ng.StatsDistKernelST(3, 3.0)
    u, z, cs = ng.RNG(9).sample_stream(k, 4)
    r = ng.RNG(9)
    for j in range(4):
        assert u[j] == r.uniform()
        assert list(z[j]) == [r.ugaussian() for _ in range(3)]
        assert cs[j] == r.chisq(3.0)


def test_handle_errors_without_device(ng):
    """Argument checks happen before any device call."""
    with pytest.raises(ng.NcgError) as e:
        ng.StatsDistVKDE(ng.StatsDistKernelGauss(0))
    assert e.value.name == "NCG_ERR_UNSUPPORTED"
    with pytest.raises(ng.NcgError) as e:
        ng.StatsDistVKDE(ng.StatsDistKernelST(3, 0.5))
    assert e.value.name == "NCG_ERR_INVALID_ARG"


_STRUCTS = ["ncg_sd_config_t", "ncg_batch_params_t", "ncg_server_config_t", "ncg_chain_desc_t",
            "ncg_step_result_t", "ncg_server_stats_t"]


def test_ctypes_structs_match_the_header(tmp_path):
    """Size and every field offset of the public structs, from the C compiler
    reading include/ncg.h, against the ctypes mirrors of the binding."""
    import shutil
    import subprocess

    from numcosmo_gb300 import _lib

    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "ncg.h"', "int main (void) {"]
    for name in _STRUCTS:
        cls = getattr(_lib, name)
        lines.append(f'printf ("{name} size %zu\\n", sizeof ({name}));')
        for f, _ in cls._fields_:
            lines.append(f'printf ("{name} {f} %zu\\n", offsetof ({name}, {f}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), "-o", str(exe), str(src)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        name, field, value = line.split()
        got[(name, field)] = int(value)
    for name in _STRUCTS:
        cls = getattr(_lib, name)
        assert got[(name, "size")] == C.sizeof(cls), name
        for f, _ in cls._fields_:
            assert got[(name, f)] == getattr(cls, f).offset, (name, f)


def test_rng_state_round_trip(ng):
    from numcosmo_gb300 import _lib

    L = _lib.load()
    r = ng.RNG(2024)
    for _ in range(700):
        r.get_u32()
    buf = C.create_string_buffer(L.ncg_rng_state_bytes())
    _lib.call("ncg_rng_get_state", r._h, buf)
    want = [r.get_u32() for _ in range(1000)]
    _lib.call("ncg_rng_set_state", r._h, buf)
    assert [r.get_u32() for _ in range(1000)] == want
    bad = C.create_string_buffer(bytes(buf.raw[:-4]) + (10 ** 6).to_bytes(4, "little"))
    with pytest.raises(ng.NcgError):
        _lib.call("ncg_rng_set_state", r._h, bad)
