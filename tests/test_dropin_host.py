"""Host side of the drop-in layer (no GPU needed): the FASTA import with Bloom de-duplication
against the reference's kept reads, and the struct layouts against the reference's headers."""
import ctypes as ct
import gzip
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, sha
import pasqual_gb300 as pq
from pasqual_gb300 import build
from oracle import port as _port

REF_SRC = _port.REFERENCE_SRC


@pytest.fixture(scope="module")
def fasta(tmp_path_factory):
    build.build()
    p = tmp_path_factory.mktemp("imp") / "import.fa"
    with gzip.open(os.path.join(GOLDEN, "import_L60.fa.gz"), "rb") as f:
        p.write_bytes(f.read())
    return str(p)


def import_fasta(width, path, L, bloom_m=36, nfunc=2):
    lib = pq.load_library(width)
    I = ct.c_uint64 if width == 64 else ct.c_uint32
    f = lib.pq_import_fasta
    f.restype = ct.c_int
    f.argtypes = [ct.c_char_p, ct.c_int, ct.c_int, ct.c_int, ct.POINTER(ct.c_void_p),
                  ct.POINTER(I), ct.POINTER(I), ct.POINTER(ct.c_char_p)]
    buf, nr, rem, err = ct.c_void_p(), I(), I(), ct.c_char_p()
    rc = f(path.encode(), L, bloom_m, nfunc, ct.byref(buf), ct.byref(nr), ct.byref(rem),
           ct.byref(err))
    if rc != 0:
        return rc, err.value.decode(), None, None
    n = nr.value * L
    arr = np.ctypeslib.as_array(ct.cast(buf, ct.POINTER(ct.c_uint8)), shape=(max(n, 1),))[:n]
    out = arr.copy().reshape(nr.value, L)
    ct.CDLL(None).free(buf)
    return 0, None, out, rem.value


@pytest.mark.parametrize("width", [32, 64])
def test_import_matches_reference(fasta, width):
    z = np.load(os.path.join(GOLDEN, "import_L60.npz"))
    rc, err, reads, removed = import_fasta(width, fasta, 60)
    assert rc == 0, err
    assert reads.shape[0] == int(z["kept%d" % width])
    assert removed == int(z["records"]) - int(z["kept%d" % width])
    assert sha(reads) == str(z["sha_reads%d" % width])


def test_import_errors(tmp_path):
    build.build()
    bad = tmp_path / "bad.fa"
    bad.write_bytes(b">a\nACGT\n>b\nACGX\n")
    rc, err, _, _ = import_fasta(32, str(bad), 4)
    assert rc == 1 and "incorrect reads file at line" in err
    short = tmp_path / "short.fa"
    short.write_bytes(b">a\nACGT\n>b\nACG\n")
    rc, err, _, _ = import_fasta(32, str(short), 4)
    assert rc == 1 and "incorrect reads file" in err
    rc, err, _, _ = import_fasta(32, str(tmp_path / "missing.fa"), 4)
    assert rc == 1 and "open reads file" in err
    # the reference CLI's argument checks (src/test.c:300-320), before any file access
    for L, m, nf, msg in ((0, 36, 2, "invalid read length (0)"), (70000, 36, 2, "invalid read length"),
                          (4, 36, 0, "invalid number of hash functions (0)"),
                          (4, 36, 6, "invalid number of hash functions (6)"),
                          (4, 0, 2, "length of bloom filter array")):
        rc, err, _, _ = import_fasta(32, str(bad), L, m, nf)
        assert rc == 1 and msg in err, (L, m, nf, err)


@pytest.mark.parametrize("width", [32, 64])
def test_import_line_semantics(tmp_path, width):
    """The whole-file import keeps the line-by-line reading of the reference (fgets into 1000
    bytes, last character of each sequence buffer dropped): a final line without a newline loses
    its last character, N reads are dropped without touching the Bloom filter, an error names
    line 2 * kept + 2, and lines of 999 or more characters take the line-by-line path."""
    build.build()
    f = tmp_path / "a.fa"
    f.write_bytes(b">a\nACGT\n>b\nccgt\n>c\nACNT\n>d\nGGGTA")       # last line: 5 chars, no newline
    rc, err, reads, removed = import_fasta(width, str(f), 4)
    assert rc == 0, err
    assert reads.tolist() == [[1, 2, 3, 4], [2, 2, 3, 4], [3, 3, 3, 4]] and removed == 1
    f.write_bytes(b">a\nACGT\n>b\nACGT\n>c\nACGX\n")                # duplicate, then a bad base
    rc, err, _, _ = import_fasta(width, str(f), 4)
    assert rc == 1 and "at line 4." in err                             # one read kept before it
    f.write_bytes(b">a\nACGT\nACGT\n>b\nACGT\n")                     # a sequence where a header belongs
    rc, err, _, _ = import_fasta(width, str(f), 4)
    assert rc == 1 and "at line 4." in err
    f.write_bytes(b">a\nACGT\n>b\n")                                  # header without a sequence line
    rc, err, _, _ = import_fasta(width, str(f), 4)
    assert rc == 1 and "at line 4." in err
    f.write_bytes(b">a\nACGT\r\n")                                    # CRLF: the CR is no base
    rc, err, _, _ = import_fasta(width, str(f), 4)
    assert rc == 1 and "at line 2." in err
    f.write_bytes(b"")
    rc, err, reads, removed = import_fasta(width, str(f), 4)
    assert rc == 0 and reads.shape[0] == 0 and removed == 0
    # a header of 1200 characters: fgets splits it, so its tail is read as the sequence line
    f.write_bytes(b">" + b"x" * 1199 + b"\nACGT\n")
    rc, err, _, _ = import_fasta(width, str(f), 4)
    assert rc == 1 and "at line 2." in err
    # NUL bytes (line by line): fgets stops nowhere special, but the C string ends at the NUL
    f.write_bytes(b">a\nACGT\n>b\nAC\x00T\n")
    rc, err, _, _ = import_fasta(width, str(f), 4)
    assert rc == 1 and "at line 4." in err
    f.write_bytes(b">a\nACGT\n>b\n\x00CGT\n")                        # a line that starts with NUL
    rc, err, _, _ = import_fasta(width, str(f), 4)
    assert rc == 1 and "at line 4." in err


def test_import_large_random_matches_line_by_line_rules(tmp_path):
    """Many records with duplicates, reverse complements, N and lowercase: the kept set is the
    reference's (golden import case) and equal for both index widths up to their own hashing."""
    build.build()
    z = np.load(os.path.join(GOLDEN, "import_L60.npz"))
    with gzip.open(os.path.join(GOLDEN, "import_L60.fa.gz"), "rb") as fh:
        text = fh.read()
    # the same records without the final newline, and with the last sequence one base longer:
    # the reference drops that base with the (absent) newline
    lines = text.rstrip(b"\n").split(b"\n")
    lines[-1] = lines[-1] + b"A"
    f = tmp_path / "nolf.fa"
    f.write_bytes(b"\n".join(lines))
    for width in (32, 64):
        rc, err, reads, removed = import_fasta(width, str(f), 60)
        assert rc == 0, err
        assert reads.shape[0] == int(z["kept%d" % width]) and sha(reads) == str(z["sha_reads%d" % width])


LAYOUT_PROG = r"""
#include <stdio.h>
#include <stddef.h>
#include HDR
#define F(T, f) printf(#T "." #f " %zu %zu\n", offsetof(T, f), sizeof(((T*)0)->f))
int main(void) {
  printf("index_t %zu\n", sizeof(IX)); printf("node_t %zu\n", sizeof(ND));
  printf("edge_t %zu\n", sizeof(ED)); printf("path_t %zu\n", sizeof(PT));
  printf("path_q_t %zu\n", sizeof(PQ)); printf("string_graph_t %zu\n", sizeof(SG));
  F(IX, bloom_array); F(IX, bloom_size); F(IX, n_hashfunc); F(IX, C); F(IX, suffix_count);
  F(IX, prefix_count); F(IX, OCC_bitmap); F(IX, OCC_bitmap_bw); F(IX, OCC_sample);
  F(IX, OCC_sample_bw); F(IX, reads_index); F(IX, reads_index_bw); F(IX, interval_start);
  F(IX, interval_end); F(IX, interval_depth); F(IX, interval_start_bw); F(IX, interval_end_bw);
  F(IX, interval_depth_bw); F(IX, read_lock); F(IX, reads); F(IX, read_len); F(IX, num_reads);
  F(IX, min_overlap); F(IX, size_bw); F(IX, offset_bw); F(IX, size_fw); F(IX, offset_fw);
  F(IX, max_size_fw); F(IX, max_size_bw);
  F(ND, edges); F(ND, path_q); F(ND, num_F); F(ND, num_B); F(ND, max_F); F(ND, max_B);
  F(ND, B_type); F(ND, F_type); F(ND, status); F(ND, marked);
  F(ED, dest); F(ED, overlap_len); F(ED, type);
  F(PT, end); F(PT, hop); F(PT, len); F(PT, end_len); F(PT, bubble_len); F(PT, trans);
  F(PT, updated); F(PT, direction); F(PT, type);
  F(PQ, path); F(PQ, max_F_endlen); F(PQ, max_B_endlen); F(PQ, max_B_len); F(PQ, max_F_len);
  F(PQ, max_F_trans); F(PQ, max_B_trans);
  F(SG, read_len); F(SG, min_overlap); F(SG, average_overlap); F(SG, num_reads); F(SG, nodes);
  return 0; }
"""


def _layout(tmp_path, hdr, defs, names, incs, extra):
    src = tmp_path / ("lay_%s.c" % names[0])
    prog = LAYOUT_PROG.replace("IX", names[0]).replace("ND", names[1]).replace("ED", names[2]) \
        .replace("PT", names[3]).replace("PQ", names[4]).replace("SG", names[5])
    prog = prog.replace('#include HDR', "\n".join('#include "%s"' % h for h in hdr))
    src.write_text(prog)
    exe = tmp_path / ("lay_%s" % names[0])
    subprocess.run(["gcc", "-std=gnu99", "-w"] + defs + ["-I" + i for i in incs] + extra +
                   [str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    # field names are the same in both; compare offsets and sizes line by line
    return [" ".join([ln.split()[0].split(".")[-1]] + ln.split()[1:]) for ln in out.splitlines()]


@pytest.mark.skipif(not os.path.isdir(REF_SRC), reason="reference headers not present")
@pytest.mark.parametrize("width", [32, 64])
def test_struct_layout_matches_reference(tmp_path, width):
    if shutil.which("gcc") is None:
        pytest.skip("no gcc")
    wdef = ["-D__INDEX_U64__"] if width == 64 else ["-D__INDEX_U32__"]
    ref = _layout(tmp_path, ["index.h", "string_graph.h"], wdef + ["-D__OPENMP__"],
                  ["index_t", "node_t", "edge_t", "path_t", "path_q_t", "string_graph_t"],
                  [REF_SRC], ["-fopenmp"])
    mine = _layout(tmp_path, ["pasqual_gb300_dropin.h"], ["-DPQ_IDX64"] if width == 64 else [],
                   ["pq_index_t", "pq_node_t", "pq_edge_t", "pq_path_t", "pq_path_q_t",
                    "pq_string_graph_t"], [os.path.join(ROOT, "include")], [])
    assert ref == mine


@pytest.mark.parametrize("width", [32, 64])
def test_reference_cli_links_and_imports(tmp_path, width):
    """The reference's own CLI objects (test.o, assemble.o, common.o, compiled from its sources
    by the oracle recipe where they are present) link against the library unchanged; run here,
    the binary imports the reads through the library, then stops at the GPU step with the
    reference's error convention (message on stderr, exit status 0) when no GPU is usable."""
    from oracle import port
    if not port.reference_buildable() or not shutil.which("gcc"):
        pytest.skip("reference sources (x86) not present")
    build.build()
    port.build(ref=True)
    objdir = os.path.join(ROOT, "oracle", "_ref", "obj_u%d" % width)
    objs = [os.path.join(objdir, o) for o in ("test.o", "assemble.o", "common.o")]
    if not all(os.path.exists(o) for o in objs):
        pytest.skip("reference objects not built")
    libdir = os.path.dirname(pq.library_path(width))
    exe = tmp_path / "pasqual_cli"
    subprocess.run(["gcc", "-fopenmp", "-o", str(exe)] + objs +
                   ["-L" + libdir, "-lpasqual_gb300_u%d" % width, "-Wl,-rpath," + libdir, "-lgomp", "-lm"],
                   check=True)
    fa = tmp_path / "r.fa"
    with gzip.open(os.path.join(GOLDEN, "import_L60.fa.gz"), "rb") as f:
        fa.write_bytes(f.read())
    z = np.load(os.path.join(GOLDEN, "import_L60.npz"))
    r = subprocess.run([str(exe), "--singlereads", str(fa), "-l", "60", "-t", "31"], cwd=str(tmp_path),
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0
    assert "Importing reads from" in r.stdout
    assert "has imported %d reads" % int(z["kept%d" % width]) in r.stdout
    import torch
    if not torch.cuda.is_available():
        assert "no usable CUDA device" in r.stderr


@pytest.mark.parametrize("width,bloom_m,nfunc", [(32, 36, 2), (64, 36, 2), (32, 6, 1), (64, 10, 3),
                                               (32, 12, 4), (64, 40, 5)])
def test_import_matches_reference_live(tmp_path, width, bloom_m, nfunc):
    """A larger generated read file (duplicates, reverse complements, N, lowercase; the Bloom
    filter also drops some unique reads as false positives, many with a short filter) imported by
    the reference itself and by the library, for every number of hash functions: the same kept
    reads, byte for byte."""
    from oracle import port
    from pasqual_gb300 import synth
    if not port.reference_buildable():
        pytest.skip("reference sources (x86) not present")
    port.build(ref=True)
    build.build()
    rng = np.random.default_rng(2024 + width)
    g = synth.genome(400000, 0.45, 0.1, (0.01, 0.02), seed=99)
    rd = synth.reads(g, 80, 40000, 0.01, seed=100)
    seqs = [bytes(synth.ACGT[r]) for r in rd]
    for i in rng.choice(len(seqs), 2000, replace=False):
        seqs.append(bytes(synth.ACGT[synth.revcomp(rd[i])]))
    for i in rng.choice(len(seqs), 1000, replace=False):
        s = bytearray(seqs[i]); s[int(rng.integers(0, 80))] = ord("N"); seqs.append(bytes(s))
    for i in rng.choice(len(seqs), 1000, replace=False):
        seqs.append(seqs[i].lower())
    order = rng.permutation(len(seqs))
    fa = tmp_path / "live.fa"
    fa.write_bytes(b"".join(b">r%d\n%s\n" % (k, seqs[j]) for k, j in enumerate(order)))
    ref = port.run_ref_dump(str(fa), 80, 41, str(tmp_path / "ref"), width=width, bloom_m=bloom_m,
                            n_hashfunc=nfunc)
    rc, err, reads, removed = import_fasta(width, str(fa), 80, bloom_m, nfunc)
    assert rc == 0, err
    assert reads.shape[0] == ref["reads"].shape[0]
    assert np.array_equal(reads, ref["reads"].reshape(reads.shape))
    assert removed == len(seqs) - reads.shape[0]
