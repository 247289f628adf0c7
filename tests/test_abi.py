"""The C ABI library builds, loads without a GPU and exports every entry
point include/sph.h declares; host-side parameter handling.  CPU only."""
import ctypes
import os
import re
import shutil
import subprocess

import pytest

from pyticles_gb300 import _abi, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "sph.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(?:int|const char \*)\s*(sph_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def libpath():
    return build.build()


def test_header_and_binding_agree():
    assert declared_symbols() == sorted(_abi.exported_symbols())


def test_library_exports_every_declared_symbol(libpath):
    lib = ctypes.CDLL(libpath)
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_library_loads_and_reports_status_strings(libpath):
    lib = _abi.lib()
    assert lib.sph_version() >= 10000
    for code, name in _abi.STATUS_NAMES.items():
        s = lib.sph_status_string(code).decode()
        assert s.startswith(name)


def test_struct_layout_matches_header(tmp_path):
    # 8 int32 + 3 doubles box + 15 doubles + int64 + collision cutoff
    assert ctypes.sizeof(_abi.SphParams) == 8 * 4 + 3 * 8 + 15 * 8 + 8 + 8
    assert _abi.SphParams.box.offset == 32
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "layout.c"
    src.write_text(
        '#include <stddef.h>\n#include <stdio.h>\n#include "sph.h"\n'
        'int main(void) { printf("%zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(sph_params),'
        ' offsetof(sph_params, box), offsetof(sph_params, thermostat_ramp_steps),'
        ' offsetof(sph_params, collision_cutoff), sizeof(sph_tuning),'
        ' offsetof(sph_tuning, cell_ratio), offsetof(sph_tuning, pair_scheme),'
        ' offsetof(sph_tuning, list_skin)); return 0; }\n')
    exe = tmp_path / "layout"
    subprocess.run([gcc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    P, T = _abi.SphParams, _abi.SphTuning
    assert got == [ctypes.sizeof(P), P.box.offset, P.thermostat_ramp_steps.offset,
                   P.collision_cutoff.offset, ctypes.sizeof(T), T.cell_ratio.offset,
                   T.pair_scheme.offset, T.list_skin.offset]


def test_make_params_defaults_follow_reference():
    p = _abi.make_params()
    assert (p.adash, p.bdash, p.kbdash) == (2.0, 0.5, 1.0)   # properties.py:18-20
    assert (p.visc_alpha, p.visc_beta) == (1.0, 0.1)          # SpamComplete eta, zeta
    assert p.sound_speed == 1.0 and p.thermalk == 1.0
    assert p.cutoff == 6.0                                     # max(h) for Lucy
    c = _abi.make_params(kernel="cubic", h_short=1.0, h_long=2.5)
    assert c.cutoff == 5.0                                     # support 2h


def test_params_roundtrip():
    p = _abi.make_params(dim=3, kernel="gaussian", box=(3, 4, 5), thermostat=True,
                         thermostat_temp=0.7, thermostat_temp_end=0.35,
                         thermostat_ramp_steps=500)
    q = _abi.params_from_dict(_abi.params_dict(p))
    assert bytes(q) == bytes(p)


def test_algorithmic_counts():
    """Work units of the rooflines: 92 flops per pair in 2D and 151 in 3D with
    heat flux; 216 unique bytes per particle for the first 2D mixed force
    launch."""
    from pyticles_gb300 import opcount
    assert opcount.flops_per_pair(2) == 92
    assert opcount.flops_per_pair(3, heat=True) == 151
    assert opcount.force_bytes_per_particle(2, 4, False) == 216
    assert opcount.force_bytes_per_step_average(2, 4) == (216 + 184) / 2


def test_autotuner_candidates_follow_the_schemes_rules():
    """Which pair schemes the tuner times (host logic only): pair lists for
    any mixed-precision group without collisions, cluster pairs for 3D
    ones, neither in FP64 or with a collision force."""
    from pyticles_gb300 import autotune
    g2 = _abi.make_params(dim=2)
    g3 = _abi.make_params(dim=3, box=(10.0, 10.0, 10.0), kernel="cubic", h_short=1.0,
                          h_long=2.0)
    gc = _abi.make_params(dim=2, collision_cutoff=0.5)   # a collision force
    assert autotune.list_candidate(g2, "mixed", []) and autotune.list_candidate(g3, "mixed", [])
    assert not autotune.list_candidate(g2, "fp64", [])
    assert not autotune.list_candidate(gc, "mixed", [])
    assert autotune.cluster_candidate(g3, "mixed", [])
    assert not autotune.cluster_candidate(g2, "mixed", [])


def test_tuning_carries_the_list_skin():
    """sph_tuning.list_skin round-trips through the binding's structure."""
    t = _abi.SphTuning(block_size=128, use_graph=1, steps_per_graph=4, rebin=0,
                       cell_ratio=0.5, pair_scheme=2, persistent=0, list_skin=0.025)
    assert (t.pair_scheme, t.list_skin) == (2, 0.025)
