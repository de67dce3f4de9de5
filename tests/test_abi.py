"""CPU tests of the boundary: libpbf.so builds, exports every symbol declared
in include/pbf.h, mirrors pbf_params' layout, and validates arguments before
touching the GPU."""
from __future__ import annotations

import ctypes
import re
import subprocess
import textwrap
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "pbf.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return re.findall(r"^\s*(?:[A-Za-z_][\w\s\*]*?[\s\*])(pbf_\w+)\s*\(", text, flags=re.M)


def test_header_declares_exported_list(pbf):
    assert declared_functions() == list(pbf.EXPORTED)


def test_library_exports_every_declared_symbol(pbf):
    L = pbf.lib()
    for name in declared_functions():
        assert hasattr(L, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", str(pbf.lib_path())], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    assert set(declared_functions()) <= exported


@pytest.mark.parametrize("cname, pyname", [("pbf_params", "PbfParams"), ("pbf_tuning", "PbfTuning"),
                                           ("pbf_step_profile", "PbfStepProfile")])
def test_struct_layout_matches_c(pbf, tmp_path, cname, pyname):
    """ctypes mirror == C struct (size and every field offset), checked by gcc."""
    cls = getattr(pbf, pyname)
    fields = [f for f, _ in cls._fields_]
    src = tmp_path / "layout.c"
    src.write_text(textwrap.dedent(f"""
        #include <stdio.h>
        #include <stddef.h>
        #include "{HEADER}"
        int main(void) {{
          printf("%zu\\n", sizeof({cname}));
          {''.join(f'printf("%zu\\n", offsetof({cname}, {f}));' for f in fields)}
          return 0;
        }}
    """))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", str(src), "-o", str(exe)], check=True)
    vals = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert vals[0] == ctypes.sizeof(cls)
    for f, off in zip(fields, vals[1:]):
        assert getattr(cls, f).offset == off, f


def test_max_particles_matches_header(pbf):
    m = re.search(r"#define PBF_MAX_PARTICLES (\d+)", HEADER.read_text())
    assert m and int(m.group(1)) == pbf.PBF_MAX_PARTICLES == 1 << 27


def test_default_params_are_the_reference_defaults(pbf):
    """fluids/FluidSystem.cpp:15-25, fluids/helper.h:4-9, fluids/Simulator.cu:174."""
    p = pbf.default_params()
    f = ctypes.c_float
    assert p.niter == 4
    assert p.g == f(9.8).value and p.h == f(0.1).value and p.dt == f(0.0083).value
    assert p.pho0 == 8000.0 and p.lambda_eps == 1000.0
    assert p.delta_q == f(0.3 * f(0.1).value).value  # 0.3 * params.h in double
    assert p.k_corr == f(0.001).value and p.n_corr == 4.0
    assert p.k_boundaryDensity == 0.0 and p.c_XSPH == 0.5
    assert list(p.up) == [0.0, 0.0, 1.0]
    assert p.lim_eps == f(1e-3).value and p.kernel_eps == f(1e-4).value and p.max_dp == f(0.1).value


def test_argument_errors_need_no_gpu(pbf):
    L = pbf.lib()
    h = ctypes.c_void_p()
    u = (ctypes.c_float * 3)(1, 1, 1)
    l = (ctypes.c_float * 3)(0, 0, 0)
    assert L.pbf_create(None, u, l, 10, ctypes.byref(h)) == pbf.PBF_ERR_INVALID_ARG
    p = pbf.default_params()
    p.niter = 0
    assert L.pbf_create(ctypes.byref(p), u, l, 10, ctypes.byref(h)) == pbf.PBF_ERR_INVALID_ARG
    assert b"niter" in L.pbf_last_error()
    p = pbf.default_params()
    p.h = float("nan")
    assert L.pbf_create(ctypes.byref(p), u, l, 10, ctypes.byref(h)) == pbf.PBF_ERR_INVALID_ARG
    p = pbf.default_params()
    bad = (ctypes.c_float * 3)(0, 1, 1)  # ulim.x == llim.x
    assert L.pbf_create(ctypes.byref(p), bad, l, 10, ctypes.byref(h)) == pbf.PBF_ERR_INVALID_ARG
    assert L.pbf_create(ctypes.byref(p), u, l, -1, ctypes.byref(h)) == pbf.PBF_ERR_INVALID_ARG
    # above the 32-bit index limit: refused before any CUDA call
    assert L.pbf_create(ctypes.byref(p), u, l, pbf.PBF_MAX_PARTICLES + 1, ctypes.byref(h)) == pbf.PBF_ERR_CAPACITY
    assert b"exceeds" in L.pbf_last_error() and h.value is None
    counts = (ctypes.c_int * 2)(pbf.PBF_MAX_PARTICLES // 2, pbf.PBF_MAX_PARTICLES // 2 + 1)
    u2 = (ctypes.c_float * 6)(1, 1, 1, 1, 1, 1)
    l2 = (ctypes.c_float * 6)(0, 0, 0, 0, 0, 0)
    assert L.pbf_batch_create(ctypes.byref(p), 2, u2, l2, counts, ctypes.byref(h)) == pbf.PBF_ERR_CAPACITY
    assert h.value is None
    # density lattice: empty or inverted boxes, 2^31 nodes (int node indices)
    fake = ctypes.c_void_p(256)  # never dereferenced: the checks fail first
    lo3, hi3 = (ctypes.c_float * 3)(0, 0, 0), (ctypes.c_float * 3)(2, 1, 1)
    for bad_lo, bad_hi, dims in (((0, 0, 0), (2, 0, 1), (4, 4, 4)), ((0, 0, 0), (2, 1, float("inf")), (4, 4, 4)),
                                 ((0, 0, 0), (2, 1, 1), (2048, 1024, 1024)), ((0, 0, 0), (2, 1, 1), (4, 0, 4))):
        d = (ctypes.c_int * 3)(*dims)
        bl, bh = (ctypes.c_float * 3)(*bad_lo), (ctypes.c_float * 3)(*bad_hi)
        assert L.pbf_density_grid(None, 0, bl, bh, d, 0.1, fake, None) == pbf.PBF_ERR_INVALID_ARG
        assert L.pbf_density_grid_backward(None, 0, bl, bh, d, 0.1, fake, None, None) == pbf.PBF_ERR_INVALID_ARG
    d = (ctypes.c_int * 3)(4, 4, 4)
    assert L.pbf_density_grid(None, 0, lo3, hi3, d, 0.0, fake, None) == pbf.PBF_ERR_INVALID_ARG
    assert L.pbf_step(None, None, None, None, None, None, 1, None) == pbf.PBF_ERR_INVALID_ARG
    assert L.pbf_set_params(None, ctypes.byref(p)) == pbf.PBF_ERR_INVALID_ARG
    assert L.pbf_destroy(None) == pbf.PBF_OK
    t = pbf.PbfTuning()
    assert L.pbf_set_tuning(None, ctypes.byref(t)) == pbf.PBF_ERR_INVALID_ARG
    assert L.pbf_get_tuning(None, ctypes.byref(t)) == pbf.PBF_ERR_INVALID_ARG
    assert L.pbf_abi_version() == 4
    assert L.pbf_status_string(pbf.PBF_ERR_CAPACITY) == b"capacity exceeded"
    with pytest.raises(pbf.PbfError) as e:
        pbf.check(pbf.PBF_ERR_TIMEOUT, "x")
    assert e.value.status == pbf.PBF_ERR_TIMEOUT


def test_create_without_gpu_reports_cuda_error(pbf):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    p = pbf.default_params()
    u = (ctypes.c_float * 3)(1, 1, 1)
    l = (ctypes.c_float * 3)(0, 0, 0)
    assert pbf.lib().pbf_create(ctypes.byref(p), u, l, 10, ctypes.byref(h)) == pbf.PBF_ERR_CUDA
    assert h.value is None


def test_cpp_facade_compiles(tmp_path):
    """The C++ Simulator facade compiles against the C ABI (no GPU call made)."""
    src = tmp_path / "facade.cpp"
    src.write_text(textwrap.dedent(f"""
        #include "{ROOT / 'pbf-cuda_gb300' / 'csrc' / 'Simulator.hpp'}"
        int use(pbf::Simulator& s, void* p, void* np, void* v, void* nv, uint32_t* iid) {{
          s.step(p, np, v, nv, iid, 10);
          pbf_params q = s.saveParams();
          s.loadParams(q);
          s.setLim({{1, 1, 1}}, {{0, 0, 0}});
          return q.niter;
        }}
    """))
    subprocess.run(["g++", "-std=c++17", "-fsyntax-only", str(src)], check=True)


def test_cpp_ssf_facade_compiles(tmp_path):
    """The C++ SSFRenderer facade compiles against the C ABI (no GPU call made)."""
    src = tmp_path / "ssf_facade.cpp"
    src.write_text(textwrap.dedent(f"""
        #include "{ROOT / 'pbf-cuda_gb300' / 'csrc' / 'SSFRenderer.hpp'}"
        int use(pbf::SSFRenderer& r, const void* pos, void* color) {{
          pbf_ssf_params p = pbf::SSFRenderer::defaults(320, 240);
          r.loadParams(p);
          r.render(pos, 10, color);
          r.setSky(nullptr, 0);
          return r.params().width;
        }}
    """))
    subprocess.run(["g++", "-std=c++17", "-fsyntax-only", str(src)], check=True)


def test_cpp_facades_throw_the_library_errors(pbf, tmp_path):
    """The C++ facades linked against libpbf.so: argument and capacity errors
    become pbf::Error with the C status before any CUDA call; without a GPU the
    constructor reports the CUDA error the same way (no exit, no abort)."""
    import torch

    csrc = ROOT / "pbf-cuda_gb300" / "csrc"
    src = tmp_path / "facade_run.cpp"
    src.write_text(textwrap.dedent(f"""
        #include <cstdio>
        #include "{csrc / 'Simulator.hpp'}"
        #include "{csrc / 'SSFRenderer.hpp'}"
        int main() {{
          pbf_params p;
          pbf_params_default(&p);
          pbf_params bad = p;
          bad.niter = 0;
          try {{ pbf::Simulator s(bad, {{1, 1, 1}}, {{0, 0, 0}}, 10); std::puts("no-throw"); }}
          catch (const pbf::Error& e) {{ std::printf("invalid %d %s\\n", (int)e.status, e.what()); }}
          try {{ pbf::Simulator s(p, {{1, 1, 1}}, {{0, 0, 0}}, PBF_MAX_PARTICLES + 1); std::puts("no-throw"); }}
          catch (const pbf::Error& e) {{ std::printf("capacity %d\\n", (int)e.status); }}
          try {{ pbf::Simulator s(p, {{1, 1, 1}}, {{0, 0, 0}}, 10); std::puts("created"); }}
          catch (const pbf::Error& e) {{ std::printf("cuda %d\\n", (int)e.status); }}
          pbf_ssf_params q = pbf::SSFRenderer::defaults(64, 48);
          q.kernel_r = 21;
          try {{ pbf::SSFRenderer r(q); std::puts("no-throw"); }}
          catch (const pbf::Error& e) {{ std::printf("ssf-invalid %d\\n", (int)e.status); }}
          return 0;
        }}
    """))
    libdir = pbf.lib_path().parent
    exe = tmp_path / "facade_run"
    subprocess.run(["g++", "-std=c++17", str(src), "-o", str(exe), f"-L{libdir}", "-lpbf", f"-Wl,-rpath,{libdir}"],
                   check=True)
    lines = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines()
    assert lines[0].startswith(f"invalid {pbf.PBF_ERR_INVALID_ARG} pbf_create") and "niter" in lines[0]
    assert lines[1] == f"capacity {pbf.PBF_ERR_CAPACITY}"
    assert lines[2] == ("created" if torch.cuda.is_available() else f"cuda {pbf.PBF_ERR_CUDA}")
    assert lines[3] == f"ssf-invalid {pbf.PBF_ERR_INVALID_ARG}"
