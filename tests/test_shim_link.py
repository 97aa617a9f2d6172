"""The reference's own driver (cpp/active_brownian.cpp) links against
libbrownian_shim unchanged: every routine it calls is defined there.  Link only
(running it needs a GPU); skipped where the reference sources are absent."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = "/root/reference/cpp"
LIB = os.path.join(ROOT, "brownian_gb300", "lib")


@pytest.mark.skipif(not os.path.exists(os.path.join(REF, "active_brownian.cpp")), reason="reference sources absent")
def test_reference_driver_links_against_the_shim(tmp_path):
    from brownian_gb300 import build
    build.build()
    exe = str(tmp_path / "a.out")
    r = subprocess.run(["g++", "-O1", "-I" + REF, "-o", exe, os.path.join(REF, "active_brownian.cpp"), "-L" + LIB,
                        "-lbrownian_shim", "-lbrownian_gb300", "-Wl,-rpath," + LIB], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
