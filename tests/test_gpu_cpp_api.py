"""The C++ drop-in classes run on the GPU: a program compiled against include/bcs/ and libsesgb.so
constructs bcs::Sesdf and bcs::Ssesdf from atoms and getAabb (sesdf/include/bcs/sesdf/sesdf.hpp:15-42,
sesdf/include/bcs/ssesdf/ssesdf.hpp:14-44), builds twice (the second time after a move), and copies
every getData() buffer, getAtomIndices() and the getD*() views to host. Each must equal, array for
array, what the Python binding of the same C ABI gives for the same atoms."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import canon
from sesdf_gb300 import SesBuild, _build, synth

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <cstdio>
#include <cstdlib>
#include <string>
#include <utility>
#include <vector>
#include <cuda_runtime_api.h>
#include "bcs/sesdf/sesdf.hpp"
#include "bcs/ssesdf/ssesdf.hpp"

static std::string g_dir;

template<class T> static void dump( const char * name, const T * device, std::size_t count )
{
    std::vector<T> host( count );
    if ( count && cudaMemcpy( host.data(), device, count * sizeof( T ), cudaMemcpyDeviceToHost ) != cudaSuccess )
        std::exit( 3 );
    FILE * f = std::fopen( ( g_dir + "/" + name + ".bin" ).c_str(), "wb" );
    if ( count )
        std::fwrite( host.data(), sizeof( T ), count, f );
    std::fclose( f );
}

static void dumpView( const char * name, const bcs::DeviceBuffer & b )
{
    const std::vector<uint8_t> host = b.toHost<uint8_t>();
    FILE * f = std::fopen( ( g_dir + "/" + name + ".bin" ).c_str(), "wb" );
    if ( !host.empty() )
        std::fwrite( host.data(), 1, host.size(), f );
    std::fclose( f );
}

static void dumpIndices( const std::vector<uint32_t> & v )
{
    FILE * f = std::fopen( ( g_dir + "/indices.bin" ).c_str(), "wb" );
    if ( !v.empty() )
        std::fwrite( v.data(), 4, v.size(), f );
    std::fclose( f );
}

int main( int argc, char ** argv )
{
    // argv: atoms file (float32 x, y, z, r), output directory, mode (full|exterior), singular probe count
    FILE * f = std::fopen( argv[ 1 ], "rb" );
    std::fseek( f, 0, SEEK_END );
    const long bytes = std::ftell( f );
    std::fseek( f, 0, SEEK_SET );
    std::vector<bcs::Vec4f> atoms( bytes / sizeof( bcs::Vec4f ) );
    if ( std::fread( atoms.data(), sizeof( bcs::Vec4f ), atoms.size(), f ) != atoms.size() )
        return 4;
    std::fclose( f );
    g_dir                  = argv[ 2 ];
    const bool     full    = std::string( argv[ 3 ] ) == "full";
    const uint32_t Q       = (uint32_t)std::strtoul( argv[ 4 ], nullptr, 10 );
    const bcs::ConstSpan<bcs::Vec4f> span { atoms.data(), atoms.size() };
    const bcs::Aabb box = bcs::getAabb( span );
    if ( full )
    {
        bcs::Sesdf first( span, box, 1.4f );
        first.build();
        if ( first.lastStatus() != 0 )
            return 10;
        bcs::Sesdf s( std::move( first ) );  // move-only, like the reference's
        s.build();
        if ( s.lastStatus() != 0 )
            return 11;
        const bcs::sesdf::SesdfData d = s.getData();
        dump( "atoms", d.atoms, d.atomNb );
        dump( "convex", d.convexPatches, d.convexPatchNb );
        dump( "sectors", d.sectors, d.sectorNb );
        dump( "segments", d.segmentPatches, d.segmentPatchNb );
        dump( "full", d.circlePatches, d.circlePatchNb );
        dump( "probe_pos", d.concavePatchesPosition, d.concavePatchNb );
        dump( "probe_ids", d.concavePatchesId, d.concavePatchNb );
        dump( "probe_nbrs", d.concavePatchesNeighbors, (std::size_t)Q * d.maxConcaveNeighbors );
        dumpIndices( s.getAtomIndices() );
        dumpView( "d_indices", s.getDAtomIndices() );
        dumpView( "d_nbr_count", s.getDAtomNeighborsCount() );
        dumpView( "d_nbr_ids", s.getDAtomNeighborsIndices() );
        dumpView( "d_status", s.getDCircleVisibilityStatus() );
        dumpView( "d_g2t", s.getDGlobalToTrimmedId() );
        const bcs::sesdf::SesdfGraphics g = s.getGraphics();
        std::printf( "%u %u %u %u %u %u %g %u %u %u\n", d.atomNb, d.sectorNb, d.segmentPatchNb, d.circlePatchNb,
                     d.concavePatchNb, (unsigned)d.maxConcaveNeighbors, d.probeRadius, g.atoms.handle,
                     g.sectorNb, (unsigned)s.getMaxNeighborPerAtom() );
    }
    else
    {
        bcs::Ssesdf first( span, box, 1.4f );
        first.build();
        if ( first.lastStatus() != 0 )
            return 10;
        bcs::Ssesdf s( std::move( first ) );
        s.build();
        if ( s.lastStatus() != 0 )
            return 11;
        const bcs::ssesdf::SsesdfData d = s.getData();
        dump( "atoms", d.atoms, d.atomNb );
        dump( "tori_pos", d.circlePosition, d.circlePatchNb );
        dump( "tori_axis", d.circleAxis, d.circlePatchNb );
        dump( "tori_vs", d.circleVs, d.circlePatchNb );
        dump( "probe_pos", d.concavePatchesPosition, d.concavePatchNb );
        dump( "probe_ids", d.concavePatchesId, d.concavePatchNb );
        dump( "probe_nbrs", d.concavePatchesNeighbors, (std::size_t)Q * d.maxConcaveNeighbors );
        dumpIndices( s.getAtomIndices() );
        dumpView( "d_indices", s.getDAtomIndices() );
        dumpView( "d_nbr_count", s.getDAtomNeighborsCount() );
        dumpView( "d_nbr_ids", s.getDAtomNeighborsIndices() );
        dumpView( "d_status", s.getDCircleVisibilityStatus() );
        const bcs::ssesdf::SsesdfGraphics g = s.getGraphics();
        std::printf( "%u %u %u %u %u %u %g %u %u %u\n", d.atomNb, 0u, 0u, d.circlePatchNb, d.concavePatchNb,
                     (unsigned)d.maxConcaveNeighbors, d.probeRadius, g.atoms.handle, 0u,
                     (unsigned)s.getMaxNeighborPerAtom() );
    }
    return 0;
}
"""


@pytest.fixture(scope="module")
def program(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    _build.build_cuda()
    d = tmp_path_factory.mktemp("cppgpu")
    src = d / "dropin.cpp"
    src.write_text(PROGRAM)
    exe = d / "dropin"
    libdir = os.path.dirname(_build.LIB)
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I", "/usr/local/cuda/include",
           str(src), "-o", str(exe), "-L", libdir, "-lsesgb", f"-Wl,-rpath,{libdir}",
           "-L", "/usr/local/cuda/lib64", "-lcudart", "-Wl,-rpath,/usr/local/cuda/lib64"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return exe


def read(d, name, dtype, width=1):
    a = np.fromfile(os.path.join(d, name + ".bin"), dtype=dtype)
    return a.reshape(-1, width) if width > 1 else a


@pytest.mark.parametrize("mode", ["full", "exterior"])
def test_dropin_classes_match_binding(program, tmp_path, mode):
    atoms = synth.globule(4000, 1003)
    with SesBuild(atoms, 1.4, mode) as g:
        g.build()
        want = g.fetch(analysis=True)
    c = want["counts"]
    f = tmp_path / "atoms.bin"
    atoms.tofile(f)
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([str(program), str(f), str(out), mode, str(c["singular_probes"])], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    fields = r.stdout.split()
    n, V, S, F, I, maxc, rp, handle, gsect, cap = fields
    assert int(n) == atoms.shape[0] and int(I) == c["probes"] and int(maxc) == 32 and float(rp) == pytest.approx(1.4)
    assert int(handle) == 0  # no graphics stack: GL handles are 0
    assert int(cap) == 128
    assert np.array_equal(read(out, "atoms", np.float32, 4), want["atoms"])
    assert np.array_equal(read(out, "probe_pos", np.float32, 4), want["probe_pos"])
    assert np.array_equal(read(out, "probe_ids", np.int32, 4), want["probe_ids"])
    Q = c["singular_probes"]
    assert np.array_equal(canon.written_probe_nbrs(read(out, "probe_nbrs", np.float32, 4), want["probe_ids"], Q),
                          canon.written_probe_nbrs(want["probe_nbrs"], want["probe_ids"], Q))
    assert np.array_equal(read(out, "indices", np.uint32), want["perm"])
    assert np.array_equal(read(out, "d_indices", np.uint32), want["perm"])
    assert np.array_equal(read(out, "d_nbr_count", np.uint32)[: atoms.shape[0]], want["nbr_count"])
    ids = read(out, "d_nbr_ids", np.uint32)[: atoms.shape[0] * 128].reshape(-1, 128)
    st = read(out, "d_status", np.uint8)[: atoms.shape[0] * 128].reshape(-1, 128)
    for i in range(atoms.shape[0]):
        k = want["nbr_count"][i]
        assert np.array_equal(ids[i, :k], want["nbr_ids"][i, :k])
        assert np.array_equal(st[i, :k], want["status"][i, :k])
    if mode == "full":
        assert int(V) == c["sectors"] and int(S) == c["segments"] and int(F) == c["full_circles"]
        assert int(gsect) == c["sectors"]
        for k in ("convex", "full"):
            assert np.array_equal(read(out, k, np.uint32, 2), want[k]), k
        assert np.array_equal(read(out, "sectors", np.float32, 4), want["sectors"])
        assert np.array_equal(read(out, "segments", np.uint32, 4), want["segments"])
        assert np.array_equal(read(out, "d_g2t", np.uint32)[: want["global_to_trimmed"].size],
                              want["global_to_trimmed"])
    else:
        assert int(F) == c["tori"]
        for k in ("tori_pos", "tori_axis", "tori_vs"):
            assert np.array_equal(read(out, k, np.float32, 4), want[k], equal_nan=True), k
