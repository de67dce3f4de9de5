"""The C oracle under AddressSanitizer and UndefinedBehaviorSanitizer: the
oracle's CPU tests run in a child process against a sanitized build of
oracle/pbf_oracle.c and oracle/ssf_oracle.c (gcc -fsanitize=address,undefined);
a failing test or any sanitizer report fails this test."""
from __future__ import annotations

import os
import subprocess
import sys
import textwrap
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
FILES = ("test_oracle.py", "test_golden.py", "test_ssf_oracle.py", "test_ssf_ref.py", "test_adjoint_oracle.py",
         "test_inverse_oracle.py", "test_density_grid_oracle.py", "test_scenes.py")


def _runtime(name: str):
    p = subprocess.run(["gcc", f"-print-file-name={name}"], capture_output=True, text=True).stdout.strip()
    return p if os.path.isabs(p) and os.path.exists(p) else None


@pytest.mark.timeout(600)
def test_oracle_is_clean_under_sanitizers(tmp_path):
    asan, ubsan = _runtime("libasan.so"), _runtime("libubsan.so")
    if not (asan and ubsan):
        pytest.skip("gcc's sanitizer runtimes are not installed")
    sys.path.insert(0, str(ROOT))
    from oracle import build_oracle

    lib = build_oracle.build_sanitized(tmp_path / "asan")
    script = tmp_path / "run.py"
    script.write_text(textwrap.dedent(f"""
        import sys
        from pathlib import Path
        sys.path.insert(0, {str(ROOT)!r})
        import oracle.build_oracle as b
        b.build = lambda *a, **k: Path({str(lib)!r})
        from oracle import oracle
        print("oracle library:", oracle.lib()._name, flush=True)
        import pytest
        sys.exit(pytest.main(["-q", "-x", "-m", "not gpu", "-p", "no:cacheprovider",
                              *{[str(ROOT / "tests" / f) for f in FILES]!r}]))
    """))
    env = dict(os.environ, LD_PRELOAD=f"{asan} {ubsan}", ASAN_OPTIONS="detect_leaks=0:halt_on_error=1",
               UBSAN_OPTIONS="print_stacktrace=1:halt_on_error=1")
    r = subprocess.run([sys.executable, str(script)], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=560)
    out = r.stdout + r.stderr
    assert r.returncode == 0, out[-3000:]
    assert "runtime error" not in out and "AddressSanitizer" not in out, out[-3000:]
    assert f"oracle library: {lib}" in out and " passed" in out
