"""The library's raw-DEFLATE decoder (BGZF blocks of BAM input) against zlib:
every block type (stored, fixed and dynamic Huffman codes), every zlib
strategy and level, many blocks on many threads, and damaged streams, which
must end in an error (or, rarely, a same-size result), never a crash."""
import zlib

import numpy as np
import pytest

from pilon_gb300 import bam


def _deflate(data, level=6, strategy=zlib.Z_DEFAULT_STRATEGY, mem=8):
    c = zlib.compressobj(level, zlib.DEFLATED, -15, mem, strategy)
    return c.compress(data) + c.flush()


def _inflate_many(payloads, threads=4):
    """Concatenates the compressed payloads and inflates them as blocks."""
    raw = b"".join(c for c, _ in payloads)
    blocks, off = [], 0
    for c, d in payloads:
        blocks.append((off, off + len(c), len(d)))
        off += len(c)
    return bytes(bam.inflate_blocks(raw, blocks, threads))


def _samples(rng):
    yield b""
    yield b"A"
    yield bytes(rng.integers(0, 256, 70000, dtype=np.uint8))                      # incompressible
    yield bytes(rng.choice(np.frombuffer(b"ACGT", np.uint8), 65000))               # 2 bits of entropy
    yield b"ACGTTGCA" * 8000                                                        # long repeats
    yield bytes(rng.integers(20, 41, 30000, dtype=np.uint8)) + b"\x00" * 20000      # quality-like, then a run
    text = b"".join(b"read%d\t%d\t60\t150M\n" % (i, i * 3) for i in range(3000))
    yield text


@pytest.mark.parametrize("level", [0, 1, 6, 9])
@pytest.mark.parametrize("strategy", [zlib.Z_DEFAULT_STRATEGY, zlib.Z_FILTERED, zlib.Z_HUFFMAN_ONLY, zlib.Z_RLE,
                                      zlib.Z_FIXED])
def test_matches_zlib(level, strategy):
    rng = np.random.Generator(np.random.PCG64(level * 10 + strategy))
    payloads = [(_deflate(d, level, strategy), d) for d in _samples(rng)]
    assert _inflate_many(payloads) == b"".join(d for _, d in payloads)


def test_small_window_and_memory_levels():
    rng = np.random.Generator(np.random.PCG64(7))
    d = bytes(rng.choice(np.frombuffer(b"ACGTN", np.uint8), 60000))
    for mem in (1, 9):
        c = _deflate(d, 9, zlib.Z_DEFAULT_STRATEGY, mem)
        assert _inflate_many([(c, d)]) == d


def test_many_blocks_any_thread_count():
    rng = np.random.Generator(np.random.PCG64(11))
    payloads = []
    for k in range(200):
        n = int(rng.integers(0, 65280))
        d = bytes(rng.choice(np.frombuffer(b"ACGT", np.uint8), n)) if k % 3 else bytes(rng.integers(0, 8, n, dtype=np.uint8))
        payloads.append((_deflate(d, int(rng.integers(0, 10))), d))
    want = b"".join(d for _, d in payloads)
    for threads in (1, 3, 16):
        assert _inflate_many(payloads, threads) == want


def test_damaged_streams_fail_cleanly():
    rng = np.random.Generator(np.random.PCG64(5))
    d = bytes(rng.choice(np.frombuffer(b"ACGT", np.uint8), 40000)) + b"TTTTTTTT" * 500
    c = _deflate(d, 6)
    with pytest.raises(ValueError):  # truncated
        _inflate_many([(c[: len(c) // 2], d)])
    with pytest.raises(ValueError):  # wrong uncompressed size
        _inflate_many([(c, d + b"x")])
    with pytest.raises(ValueError):  # block type 3
        _inflate_many([(b"\x07" + c[1:], d)])
    for k in range(300):  # flipped bits: an error, or by chance output of the stated size
        bad = bytearray(c)
        for _ in range(int(rng.integers(1, 4))):
            i = int(rng.integers(0, len(bad)))
            bad[i] ^= 1 << int(rng.integers(0, 8))
        try:
            out = _inflate_many([(bytes(bad), d)])
            assert len(out) == len(d)
        except ValueError:
            pass
    for k in range(100):  # random bytes
        junk = bytes(rng.integers(0, 256, int(rng.integers(1, 500)), dtype=np.uint8))
        try:
            _inflate_many([(junk, b"\0" * 1000)])
        except ValueError:
            pass
