"""The drop-in executables' file helpers (muca_gb300/cli/cli_common.h) on
the host, compiled into a small program: the histogram dump in the format
of the reference's commented-out output (muca_delta_multigpu.cu:528-541),
one line "i lnW[i] H[i]" per bin with lnW to 10 significant digits, as
the weight files (:490-492)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROG = r'''
#include "cli_common.h"
int main(int argc, char **argv)
{
    std::vector<double> w = {0.0, -1.5, 1234.56789012345, -9.87654321e-7, 3.0e12};
    std::vector<uint64_t> h = {0, 1, 18446744073709551615ull, 42, 7};
    std::string why;
    if (!cli::write_hist_dump(argv[1], w, h, why)) { std::fprintf(stderr, "%s\n", why.c_str()); return 1; }
    std::vector<uint64_t> h4(4);
    if (cli::write_hist_dump(argv[2], w, h4, why)) return 2;  // sizes differ: refused
    std::printf("%s\n", why.c_str());
    return 0;
}
'''


@pytest.fixture(scope="module")
def prog(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("no g++")
    d = tmp_path_factory.mktemp("clifiles")
    src = d / "t.cpp"
    src.write_text(PROG)
    exe = d / "t"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I",
                    os.path.join(ROOT, "muca_gb300", "cli"), str(src), "-o", str(exe)], check=True)
    return str(exe)


def test_hist_dump_format(prog, tmp_path):
    out, bad = tmp_path / "dump.txt", tmp_path / "bad.txt"
    r = subprocess.run([prog, str(out), str(bad)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "5 weights for 4 bins" in r.stdout
    lines = out.read_text().splitlines()
    w = [0.0, -1.5, 1234.56789012345, -9.87654321e-7, 3.0e12]
    h = [0, 1, 18446744073709551615, 42, 7]
    assert len(lines) == 5
    for i, line in enumerate(lines):
        a, b, c = line.split(" ")
        assert int(a) == i
        assert b == "%.10g" % w[i]  # ostream with setprecision(10), default float format
        assert int(c) == h[i]
    assert lines[2].split()[1] == "1234.56789"


def test_hist_dump_unwritable_path(prog, tmp_path):
    r = subprocess.run([prog, str(tmp_path / "no" / "such" / "dir.txt"), str(tmp_path / "b.txt")],
                       capture_output=True, text=True)
    assert r.returncode == 1 and "cannot be opened" in r.stderr
