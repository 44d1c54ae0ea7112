"""The extended tracer's double-float pair (EM_PREC_DF64) restated in C99
on the CPU (tests/df_pair_check.c): its accuracy claim, about 2^-42 relative
per term (within 1e-12 here, 4.8e-13 measured), against a long-double
evaluation, with the rsqrt estimate perturbed by up to 1.3e-7."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_double_float_pair_accuracy(tmp_path):
    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = tmp_path / "df_pair_check"
    subprocess.check_call([cc, "-std=c99", "-O2", "-ffp-contract=off",
                           os.path.join(ROOT, "tests", "df_pair_check.c"),
                           "-o", str(exe), "-lm"])
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
