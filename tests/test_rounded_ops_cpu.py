"""CPU restatement of the exact arithmetic's branch-free rounded operations
(tests/rounded_ops_check.c): the quotient step rounds correctly from a
correctly rounded reciprocal (Markstein's theorem, 2e8 random quotients
against the double quotient rounded to float), and the one-step reciprocal
and root reproduce a correctly rounded start; how starts 1-2 ulp off fare is
reported, since exactness there rests on the device's approximations, which
the library checks on the device before it uses them."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_rounded_ops_restatement(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = str(tmp_path / "rounded_ops_check")
    subprocess.check_call([cc, "-O2", "-ffp-contract=off", "-std=c99", "-o", exe,
                           os.path.join(HERE, "rounded_ops_check.c"), "-lm"])
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count("ok ") == 2, r.stdout
