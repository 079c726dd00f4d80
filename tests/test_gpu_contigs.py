"""contigs.fa from the GPU path, through the reference's own CLI.

The reference's CLI sources that stay on the host (test.c, assemble.c, common.c and their
headers, src/test.c:364-391, src/assemble.c:2876-3021) are compiled unchanged and linked against
this library, which serves construct_index and construct_string_graph (suffix sorts, FM-indexes
and overlap search on the GPU, node construction on the host).  The binary runs
`--singlereads FILE -l L -t T` on each workload-size case's reads, with OMP_NUM_THREADS=1 for the
assembly stage, and its contigs.fa must have the SHA-256 of the contigs.fa the reference's own
binary wrote from the same FASTA (tests/golden/large/, made by tests/golden/make_golden.py).

The CLI sources are staged from the reference tree by `make -C oracle stage` (run by the build
where the tree is present) into oracle/_ref/cli_src/, a folder that is not part of the
repository; without them the test is skipped.  They are compiled with x86 semantics where the
two hosts differ (signed char, no contraction of floating-point multiply-adds) so that an Arm
host computes what the reference computes on x86.
"""
import hashlib
import os
import subprocess

import pytest

from conftest import ROOT, large_cases, large_kept_reads, load_large
import pasqual_gb300 as pq

pytestmark = pytest.mark.gpu

CLI_SRC = os.path.join(ROOT, "oracle", "_ref", "cli_src")
CFLAGS = ["-O2", "-std=gnu99", "-fopenmp", "-D__OPENMP__", "-D__TIMING__", "-fsigned-char",
          "-ffp-contract=off", "-w"]


@pytest.fixture(scope="module")
def cli(tmp_path_factory):
    """The reference's CLI linked against libpasqual_gb300_u32/u64: {width: path}."""
    srcs = [os.path.join(CLI_SRC, s) for s in ("test.c", "assemble.c", "common.c")]
    if not all(os.path.exists(s) for s in srcs):
        pytest.skip("the reference's CLI sources are not staged (make -C oracle stage)")
    out = tmp_path_factory.mktemp("cli")
    exes = {}
    for width in (32, 64):
        libdir = os.path.dirname(pq.library_path(width))
        exe = str(out / ("pasqual_gb300_cli_u%d" % width))
        subprocess.run(["gcc"] + CFLAGS + ["-D__INDEX_U%d__" % width, "-I" + CLI_SRC, "-o", exe] + srcs +
                       ["-L" + libdir, "-lpasqual_gb300_u%d" % width, "-Wl,-rpath," + libdir, "-lgomp",
                        "-lm"], check=True)
        exes[width] = exe
    return exes


@pytest.mark.parametrize("name", large_cases())
def test_contigs_from_gpu_path_match_reference(tmp_path, cli, name):
    g = load_large(name)
    _, fa = large_kept_reads(g, tmp_path)
    run = tmp_path / "run"
    run.mkdir()
    r = subprocess.run([cli[int(g["width"])], "--singlereads", fa, "-l", str(int(g["read_len"])),
                        "-t", str(int(g["t"]))], cwd=str(run), capture_output=True, text=True,
                       timeout=1200, env=dict(os.environ, OMP_NUM_THREADS="1"))
    # the reference's error convention is a message on stderr and exit status 0 (src/common.h:87-94)
    assert r.returncode == 0 and (run / "contigs.fa").exists(), r.stderr[-2000:]
    contigs = (run / "contigs.fa").read_bytes()
    assert contigs.count(b">") == int(g["contigs"])
    assert hashlib.sha256(contigs).hexdigest() == str(g["sha_contigs"])
