"""The reference's own driver (cpp/active_brownian.cpp) links against
libbrownian_shim unchanged: every routine it calls is defined there.  Link only
(running it needs a GPU); skipped unless BROWNIAN_REFERENCE names a reference
checkout (the directory holding cpp/)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(os.environ.get("BROWNIAN_REFERENCE", ""), "cpp")
LIB = os.path.join(ROOT, "brownian_gb300", "lib")


@pytest.mark.skipif(not os.path.exists(os.path.join(REF, "active_brownian.cpp")), reason="BROWNIAN_REFERENCE unset or without cpp/")
def test_reference_driver_links_against_the_shim(tmp_path):
    from brownian_gb300 import build
    build.build()
    exe = str(tmp_path / "a.out")
    r = subprocess.run(["g++", "-O1", "-I" + REF, "-o", exe, os.path.join(REF, "active_brownian.cpp"), "-L" + LIB,
                        "-lbrownian_shim", "-lbrownian_gb300", "-Wl,-rpath," + LIB], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
