"""CPU checks of the boundary: the library loads and exports every symbol the
header declares; ctypes struct layouts match the header; host-side validation."""
import ctypes as C
import os
import re

import pytest

from cgenie_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    names = set()
    for h in sorted(f for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h")):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(gb_(?:go|ens|bg|ea|mo|rs|ts|tr)_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


def test_library_builds_and_exports_all_header_symbols():
    from cgenie_gb300 import build, goldstein
    path = build.build()
    lib = C.CDLL(path)
    names = header_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(goldstein.EXPORTED) == names


def test_struct_layouts():
    assert C.sizeof(abi.GbDims) == 16
    # 2+5 doubles, 3 doubles, 8 int32, mldpebuoycoeff
    assert C.sizeof(abi.GbParams) == (7 + 3) * 8 + 8 * 4 + 8
    # 19 pointers, dphi and rdphi, 3 pointers of the mixed-layer scheme
    assert C.sizeof(abi.GbGrid) == 19 * 8 + 2 * 8 + 3 * 8
    assert C.sizeof(abi.GbEnsTuning) == 24
    assert C.sizeof(abi.GbBgDims) == 24
    assert C.sizeof(abi.GbBgParams) == 24
    assert C.sizeof(abi.GbEaDims) == 8
    assert C.sizeof(abi.GbEaParams) == 8 + 14 * 8
    assert C.sizeof(abi.GbEaGrid) == 7 * 8
    assert C.sizeof(abi.GbRsCalendar) == 4 * 4 + 8
    from cgenie_gb300 import momentum
    assert C.sizeof(momentum.GbMoDims) == 24
    assert C.sizeof(momentum.GbMoParams) == 24
    assert C.sizeof(momentum.GbMoGrid) == 26 * 8


def test_errstr_without_gpu():
    from cgenie_gb300 import build, goldstein
    build.build()
    lib = goldstein.load_library()
    assert lib.gb_go_errstr(0) == b"ok"
    assert lib.gb_go_errstr(abi.GB_GO_EINVAL) == b"invalid argument"
    assert lib.gb_go_errstr(-99) == b"unknown error"


def test_oracle_header_cites_reference():
    src = open(os.path.join(ROOT, "oracle", "goldstein_oracle.c")).read()
    assert "ORACLE -- test infrastructure only" in src
    assert "goldstein.f90:2436-2642" in src
    assert "parity unpinned" in src


def test_autotune_candidates_start_with_planner_choice():
    from cgenie_gb300 import autotune
    for shape in [(18, 18), (36, 36), (37, 23)]:
        c = autotune.candidates(*shape)
        assert c[0] == (0, 0)
        assert all(64 <= tx * ty <= 128 for tx, ty in c[1:])
    assert autotune.lookup({"36x36x16": [12, 9, 1.0]}, 36, 36, 16) == (12, 9)
    assert autotune.lookup({}, 36, 36, 16) is None


def test_host_memory_calls_refuse_bad_arguments_without_gpu():
    """gb_ens_host_alloc / gb_ens_host_free validate their arguments before any CUDA call:
    a zero size or NULL result pointer, and a pointer the allocator did not return, are
    GB_GO_EINVAL."""
    from cgenie_gb300 import build, goldstein
    build.build()
    lib = goldstein.load_library()
    p = C.c_void_p()
    assert lib.gb_ens_host_alloc(C.c_size_t(0), C.byref(p)) == abi.GB_GO_EINVAL
    assert lib.gb_ens_host_alloc(C.c_size_t(64), None) == abi.GB_GO_EINVAL
    buf = (C.c_char * 64)()
    assert lib.gb_ens_host_free(C.cast(buf, C.c_void_p)) == abi.GB_GO_EINVAL
    assert lib.gb_ens_host_free(None) == abi.GB_GO_EINVAL


def test_trace_calls_without_gpu():
    """The ITT-shaped tracing calls (include/gb_trace.h) work without a GPU or a profiler:
    domains are one per name, NULL names are refused, tasks nest and close, and the collection
    window calls report the missing device instead of failing."""
    from cgenie_gb300 import build, goldstein
    build.build()
    L = goldstein.load_library()
    d = L.gb_tr_domain_create(b"genie")
    assert d and L.gb_tr_domain_create(b"genie") == d and L.gb_tr_domain_create(b"other") != d
    assert not L.gb_tr_domain_create(None) and not L.gb_tr_domain_create(b"")
    assert not L.gb_tr_string_handle_create(None)
    step, status = L.gb_tr_string_handle_create(b"timestep"), L.gb_tr_string_handle_create(b"status")
    assert step and status
    L.gb_tr_task_begin(d, step)
    L.gb_tr_task_begin(d, status)
    L.gb_tr_task_end(d)
    L.gb_tr_task_end(d)
    L.gb_tr_task_begin(None, None)   # the library's own domain, unnamed
    L.gb_tr_task_end(None)
    assert L.gb_tr_resume() in (abi.GB_GO_OK, abi.GB_GO_ECUDA)
    assert L.gb_tr_pause() in (abi.GB_GO_OK, abi.GB_GO_ECUDA)
