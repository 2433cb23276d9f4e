"""The C++ drop-in headers compile against the library, and bcs::load (include/bcs/core/loader.hpp, the
reference's loader for MMTF files) reads what the Python reader reads. Host only: nothing here touches a GPU."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from sesdf_gb300 import _build, mmtf
from test_mmtf import minimal_document

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <cstdio>
#include "bcs/core/loader.hpp"
#include "bcs/sesdf/sesdf.hpp"
#include "bcs/ssesdf/ssesdf.hpp"
int main( int argc, char ** argv )
{
    try
    {
        const bcs::Molecule m = bcs::load( argv[ 1 ] );
        std::printf( "%zu\n", m.size() );
        for ( const bcs::Vec4f & a : m )
            std::printf( "%.9g %.9g %.9g %.9g\n", a.x, a.y, a.z, a.w );
        const bcs::Aabb box = bcs::getAabb( bcs::ConstSpan<bcs::Vec4f> { m.data(), m.size() } );
        std::printf( "%.9g %.9g\n", box.min.x, box.max.x );
    }
    catch ( const std::exception & e )
    {
        std::printf( "error %s\n", e.what() );
        return 2;
    }
    return 0;
}
"""


@pytest.fixture(scope="module")
def program(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    _build.build_cuda()
    d = tmp_path_factory.mktemp("cpp")
    src = d / "load.cpp"
    src.write_text(PROGRAM)
    exe = d / "load"
    libdir = os.path.dirname(_build.LIB)
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I", "/usr/local/cuda/include",
           str(src), "-o", str(exe), "-L", libdir, "-lsesgb", f"-Wl,-rpath,{libdir}",
           "-L", "/usr/local/cuda/lib64", "-lcudart", "-Wl,-rpath,/usr/local/cuda/lib64"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return exe


def test_load_matches_python_reader(program, tmp_path):
    doc = minimal_document(("N", "c", "SE", "Q"), (1234, -5678, 32766, 1))
    f = tmp_path / "m.mmtf"
    f.write_bytes(doc)
    r = subprocess.run([str(program), str(f)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = r.stdout.split("\n")
    n = int(lines[0])
    got = np.array([[float(v) for v in ln.split()] for ln in lines[1:1 + n]], np.float32)
    want = mmtf.load_bytes(doc)
    assert np.array_equal(got, want)
    lo, hi = (float(v) for v in lines[1 + n].split())
    assert lo == np.float32(want[:, 0] - want[:, 3]).min() and hi == np.float32(want[:, 0] + want[:, 3]).max()


def test_load_reports_errors(program, tmp_path):
    f = tmp_path / "bad.mmtf"
    f.write_bytes(b"\x80")
    r = subprocess.run([str(program), str(f)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and r.stdout.startswith("error")
    r = subprocess.run([str(program), str(tmp_path / "missing.mmtf")], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "cannot open" in r.stdout
