"""The FASTA import against an independent restatement of the reference's reading, on many small
random files full of edge cases: fgets into 1000 bytes, the last character of each sequence buffer
dropped, C-string lengths (a NUL byte ends the line), base and N classes, the error line number
2 * kept + 2, and the Bloom filter's five hashes in index-width arithmetic
(src/index.c:145-405, src/bloom.c:18-135)."""
import numpy as np
import pytest

from pasqual_gb300 import build
from test_dropin_host import import_fasta

CODE = {ord(c): i + 1 for i, c in enumerate("ACGT")}
CODE.update({ord(c): i + 1 for i, c in enumerate("acgt")})


def fgets_chunks(data: bytes, size: int = 1000):
    """What repeated fgets(buf, size, fp) returns: at most size-1 bytes, up to and with '\\n'."""
    out, i = [], 0
    while i < len(data):
        j = data.find(b"\n", i, i + size - 1)
        end = j + 1 if j >= 0 else min(len(data), i + size - 1)
        out.append(data[i:end])
        i = end
    return out


def cstr(b: bytes) -> bytes:
    k = b.find(b"\0")
    return b if k < 0 else b[:k]


def hashes(codes, m, width, nf):
    mask = (1 << width) - 1
    h = [0] * 5
    for c in codes:
        h[0] = (h[0] ^ (((h[0] << 5) + (h[0] >> 2) + c) & mask)) & mask
        h[1] = (c + (h[1] << 6) + (h[1] << 16) - h[1]) & mask
        h[2] = (h[2] + c) & mask
        h[3] = h[3] ^ c
        h[4] = (33 * h[4] + c) & mask
    return [x % m for x in h[:nf]]


def model_import(data: bytes, L: int, bloom_m: int, nf: int, width: int):
    chunks = fgets_chunks(data)
    records = sum(1 for c in chunks if c[:1] == b">")
    m = (records * bloom_m) & ((1 << width) - 1)
    bits = set()
    kept, removed = [], 0
    it = iter(chunks)
    for hdr in it:
        if hdr[:1] != b">":
            return ("err", 2 * len(kept) + 2)
        seq = next(it, None)
        if seq is None:
            return ("err", 2 * len(kept) + 2)
        s = cstr(seq)
        if len(s) == 0:
            return ("err", 2 * len(kept) + 2)
        s = s[:-1]
        if len(s) != L:
            return ("err", 2 * len(kept) + 2)
        fw, with_n = [], False
        for ch in s:
            if ch in CODE:
                fw.append(CODE[ch])
            elif ch in (ord("N"), ord("n")):
                with_n = True
                fw.append(ord("N"))
            else:
                return ("err", 2 * len(kept) + 2)
        if with_n:
            removed += 1
            continue
        rc = [5 - c for c in reversed(fw)]
        hv = hashes(fw, m, width, nf)
        if all(x in bits for x in hv) or all(x in bits for x in hashes(rc, m, width, nf)):
            removed += 1
            continue
        bits.update(hv)
        kept.append(fw)
    return ("ok", np.array(kept, np.uint8).reshape(len(kept), L), removed)


def random_file(rng, L):
    bases = rng.integers(0, 4, (int(rng.integers(1, 40)), L))
    noisy = rng.random() < 0.5                                      # half the files hold errors
    recs = []
    for k in range(int(rng.integers(0, 60))):
        b = bases[int(rng.integers(0, len(bases)))]
        if rng.random() < 0.15:
            b = 3 - b[::-1]                                        # reverse complement
        seq = bytearray(b"ACGT"[x] for x in b)
        if rng.random() < 0.2:
            seq = seq.lower() if rng.random() < 0.5 else bytearray(
                c | (0x20 if rng.random() < 0.5 else 0) for c in seq)
        if rng.random() < 0.05:
            seq[int(rng.integers(0, L))] = ord("N")
        hdr, nl = b">r%d" % k, b"\n"
        r = rng.random() if noisy else 1.0
        if r < 0.02:
            seq[int(rng.integers(0, L))] = int(rng.choice(list(b"XRn>- \r")))
        elif r < 0.03:
            seq = seq[: int(rng.integers(0, L))]                    # short
        elif r < 0.04:
            seq = seq + b"A"                                        # long
        elif r < 0.05:
            seq[int(rng.integers(0, L))] = 0                        # NUL byte
        elif r < 0.06:
            hdr = b">" + b"h" * int(rng.integers(990, 1010))       # around the fgets limit
        elif r < 0.07:
            hdr = b"r%d" % k                                        # no '>'
        elif r < 0.08:
            nl = b"\r\n"
        recs.append(hdr + b"\n" + bytes(seq) + nl)
    data = b"".join(recs)
    if data and rng.random() < 0.2:
        data = data[:-1]                                            # no final newline
    if rng.random() < 0.05:
        data += b"\n"                                               # a trailing empty line
    return data


@pytest.mark.parametrize("width", [32, 64])
def test_import_fuzz_against_restatement(tmp_path, width):
    build.build()
    rng = np.random.default_rng(4242 + width)
    f = tmp_path / "f.fa"
    n_ok = n_err = 0
    for case in range(1000):
        L = int(rng.choice([1, 3, 8, 20, 60]))
        bloom_m = int(rng.choice([1, 2, 5, 36]))
        nf = int(rng.integers(1, 6))
        data = random_file(rng, L)
        f.write_bytes(data)
        want = model_import(data, L, bloom_m, nf, width)
        rc, err, reads, removed = import_fasta(width, str(f), L, bloom_m, nf)
        if want[0] == "err":
            n_err += 1
            assert rc == 1 and err == "incorrect reads file at line %d.\n" % want[1], (case, err, want)
        else:
            n_ok += 1
            assert rc == 0, (case, err)
            assert reads.shape == want[1].shape and np.array_equal(reads, want[1]), case
            assert removed == want[2], case
    assert n_ok > 300 and n_err > 300


@pytest.mark.parametrize("width", [32, 64])
def test_restatement_matches_reference(tmp_path, width):
    """The restatement above pinned to the reference's own import (its construct_index, compiled
    by the oracle recipe) on random edge-case files: the same error, or the same numbers of kept
    and removed reads (and the same bytes where the reference's sort of so few reads completes)."""
    import os
    import subprocess
    from oracle import port
    if not port.reference_buildable():
        pytest.skip("reference sources (x86) not present")
    port.build(ref=True)
    exe = os.path.join(port.REF, "ref_dump_u%d" % width)
    rng = np.random.default_rng(77 + width)
    f = tmp_path / "f.fa"
    compared = 0
    while compared < 40:
        L = int(rng.choice([20, 60]))
        bloom_m, nf = int(rng.choice([1, 2, 5, 36])), int(rng.integers(1, 6))
        data = random_file(rng, L)
        if b"\0" in data:
            continue                  # the reference writes before its buffer on a NUL-led line
        want = model_import(data, L, bloom_m, nf, width)
        if want[0] == "ok" and want[1].shape[0] < 2:
            continue                  # the reference's sort needs reads to sort
        f.write_bytes(data)
        out = tmp_path / ("d%d" % compared)
        r = subprocess.run([exe, str(f), str(L), str(L - 5), str(out), "1", str(bloom_m), str(nf)],
                           capture_output=True, text=True, timeout=120)
        if want[0] == "err":
            assert "incorrect reads file at line %d." % want[1] in r.stderr, (r.stderr, want)
        else:
            # the import's own report; the reference's sort may then fail on a few reads
            assert "has imported %d reads (removed %d duplicate reads)" % (want[1].shape[0], want[2]) \
                in r.stdout, (r.stdout, want[1].shape, want[2])
            if r.returncode == 0:
                got = np.fromfile(os.path.join(str(out), "reads.bin"), np.uint8)
                assert np.array_equal(got, want[1].reshape(-1))
        compared += 1
