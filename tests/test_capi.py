"""CPU tests of the C ABI boundary: the library builds for sm_103a, loads,
exports every symbol include/fvs_gpu.h declares, and validates arguments
before touching a device.  No compute is launched here."""
import ctypes as C

import pytest


@pytest.fixture(scope="module")
def capi():
    from finitevolumesolver_gb300 import _capi, build
    build.build()
    return _capi


def test_exports_every_header_symbol(capi):
    L = capi.load()
    names = capi.header_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_no_gpu_reports_no_device(capi):
    L = capi.load()
    if L.fvs_device_count() > 0:
        pytest.skip("a GPU is visible")
    import finitevolumesolver_gb300 as f
    g = capi.GridDesc()
    g.rank = 1
    g.n[0], g.n[1], g.n[2] = 8, 1, 1
    g.bc[0] = 1
    g.dx[0] = 0.1
    m = f.make_method()
    h = C.c_void_p()
    assert L.fvs_solver_create(C.byref(g), C.byref(m), C.byref(h)) == capi.FVS_ERR_NO_DEVICE
    with pytest.raises(f.FvsError):
        f.Solver([8], [0.1], "transmissive")
    h2 = C.c_void_p()
    assert L.fvs_patch_ctx_create(C.byref(h2)) == capi.FVS_ERR_NO_DEVICE
    # both stable-dt entry points report the missing device the same way
    out = C.c_double(0.0)
    b = f.box([0, 0], [8, 8])
    for fn in (L.fvs_compute_stable_dt, L.fvs_compute_stable_dt_noalloc):
        assert fn(C.byref(m), 2, 1, b, 0.1, 0, 0, C.byref(out), None) == \
            capi.FVS_ERR_NO_DEVICE


def test_argument_validation_before_device(capi):
    import finitevolumesolver_gb300 as f
    L = capi.load()
    m = f.make_method()
    # cell box that does not cover the MUSCL stencil of the faces
    r = L.fvs_compute_numeric_fluxes(C.byref(m), 1, 1, f.box([0], [5]), 1, f.box([0], [5]), 0.1,
                                     0.1, 0, None)
    assert r == capi.FVS_ERR_INVALID
    assert b"stencil" in L.fvs_last_error()
    # direction out of range
    r = L.fvs_compute_numeric_fluxes(C.byref(m), 2, 1, f.box([0, 0], [5, 5]), 1,
                                     f.box([-2, -2], [7, 7]), 0.1, 0.1, 2, None)
    assert r == capi.FVS_ERR_INVALID
    # unknown limiter
    m2 = f.make_method(limiter=7)
    r = L.fvs_compute_numeric_fluxes(C.byref(m2), 1, 1, f.box([0], [5]), 1, f.box([-2], [7]),
                                     0.1, 0.1, 0, None)
    assert r == capi.FVS_ERR_INVALID
    # update: face box too small
    r = L.fvs_update_conservatively(1, f.box([0], [4]), 1, f.box([0], [4]), 1, f.box([0], [4]),
                                    3, 0.1, 0.1, 0, None)
    assert r == capi.FVS_ERR_INVALID
    # the allocation-free stable dt checks its arguments like the allocating one
    for fn in (L.fvs_compute_stable_dt, L.fvs_compute_stable_dt_noalloc):
        out = C.c_double(0.0)
        assert fn(C.byref(m2), 1, 1, f.box([0], [8]), 0.1, 0, 0, C.byref(out), None) == \
            capi.FVS_ERR_INVALID  # unknown limiter
        m3 = f.make_method(precision="fp64_exact")
        m3.precision = 9
        assert fn(C.byref(m3), 1, 1, f.box([0], [8]), 0.1, 0, 0, C.byref(out), None) == \
            capi.FVS_ERR_INVALID  # unknown precision
        assert fn(C.byref(m), 1, 1, f.box([0], [8]), 0.1, 0, 2, C.byref(out), None) == \
            capi.FVS_ERR_INVALID  # unknown window rule
    # bad grid
    g = capi.GridDesc()
    g.rank = 2
    g.n[0], g.n[1], g.n[2] = 8, 8, 4
    h = C.c_void_p()
    assert L.fvs_solver_create(C.byref(g), C.byref(m), C.byref(h)) == capi.FVS_ERR_INVALID


def test_method_defaults_match_reference(capi):
    import finitevolumesolver_gb300 as f
    m = f.make_method()
    # include/fub/NewtonIteration.hpp:29-30, PerfectGas.hpp:209
    assert m.max_iterations == 5000 and m.tolerance == 1e-7 and m.gamma == 1.4
    assert f.FluxMethod(f.PerfectGas(2)).GetStencilWidth() == 2
    assert f.FluxMethod(f.PerfectGas(2), "hlle").GetStencilWidth() == 1


def test_no_template_shared_between_fma_and_no_fma_units(capi):
    """A template instantiated with the same arguments in a -fmad=false unit
    and in an FMA unit is one weak symbol: the linker keeps one copy, so one
    flavour would silently run the other's kernels.  Every such template
    carries a flavour argument; no weak symbol of the library's namespace is
    defined by units compiled with different -fmad flags."""
    import shutil
    import subprocess

    from finitevolumesolver_gb300 import build

    nm = shutil.which("nm")
    if nm is None:
        pytest.skip("nm not available")
    owners = {}
    for src, flags in build.UNITS:
        obj = build.BUILD_DIR / (src.rsplit(".", 1)[0] + ".o")
        if not obj.exists():
            pytest.skip(f"{obj.name} not built")
        out = subprocess.run([nm, "-C", "--defined-only", str(obj)], capture_output=True,
                             text=True, check=True).stdout
        nofma = "-fmad=false" in flags
        for line in out.splitlines():
            parts = line.split(" ", 2)
            if len(parts) == 3 and parts[1] in ("W", "V") and "fvs::" in parts[2]:
                owners.setdefault(parts[2], set()).add(nofma)
    clashes = sorted(sym for sym, kinds in owners.items() if len(kinds) > 1)
    assert not clashes, clashes[:5]
