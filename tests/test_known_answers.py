"""The oracle against the reference's own known-answer vectors: the codec
specifications' worked examples (src/openzl/codecs/*/spec.md) and the
tokenize node tests (tests/codecs/test_tokenize.cpp:108-178)."""
import numpy as np

from oracle import oracle

TR_DELTA, TR_ZIGZAG, TR_TSPLIT, TR_BITPACK_INT = 1, 3, 4, 28
S, ST, N = oracle.TYPE_SERIAL, oracle.TYPE_STRUCT, oracle.TYPE_NUMERIC


def test_delta_spec_example():
    # codecs/delta/spec.md:12: header 2, deltas {1, 1, 2} -> {2, 3, 4, 6}
    for w, dt in [(1, np.uint8), (2, np.uint16), (4, np.uint32), (8, np.uint64)]:
        hdr = np.array([2], dt).tobytes()
        out, t, ow, n = oracle.decode_transform(TR_DELTA, hdr, [(N, w, np.array([1, 1, 2], dt).tobytes())])
        assert t == N and ow == w and n == 4
        assert np.frombuffer(out.tobytes(), dt).tolist() == [2, 3, 4, 6]


def test_zigzag_spec_example():
    # codecs/zigzag/spec.md:10: {1, 3, 4} -> {-1, -2, 2}
    for w, dt, st in [(1, np.uint8, np.int8), (2, np.uint16, np.int16), (4, np.uint32, np.int32),
                      (8, np.uint64, np.int64)]:
        out, t, ow, n = oracle.decode_transform(TR_ZIGZAG, b"", [(N, w, np.array([1, 3, 4], dt).tobytes())])
        assert np.frombuffer(out.tobytes(), st).tolist() == [-1, -2, 2]


def test_bitpack_spec_example():
    # codecs/bitpack/spec.md:14-25: stream |11111010|11011000|11011100|, header
    # |01000010| (nbBits 3, width 2) -> {2, 7, 3, 4, 5, 1, 7, 6}; a second
    # header byte 2 drops the last two -> {2, 7, 3, 4, 5, 1}
    stream = bytes([0b11111010, 0b11011000, 0b11011100])
    out, t, ow, n = oracle.decode_transform(TR_BITPACK_INT, bytes([0b01000010]), [(S, 1, stream)])
    assert ow == 2 and np.frombuffer(out.tobytes(), np.uint16).tolist() == [2, 7, 3, 4, 5, 1, 7, 6]
    out, t, ow, n = oracle.decode_transform(TR_BITPACK_INT, bytes([0b01000010, 2]), [(S, 1, stream)])
    assert np.frombuffer(out.tobytes(), np.uint16).tolist() == [2, 7, 3, 4, 5, 1]


def test_transpose_spec_example():
    # codecs/transpose/spec.md: {"1234", "abcd"} -> {"1a", "2b", "3c", "4d"}
    out, t, ow, n = oracle.decode_transform(TR_TSPLIT, b"", [(S, 1, b"1234"), (S, 1, b"abcd")])
    assert t == ST and ow == 2 and n == 4 and out.tobytes() == b"1a2b3c4d"


def test_tokenize_known_answers():
    # tests/codecs/test_tokenize.cpp:108-178
    for dt in (np.uint8, np.int16, np.int32, np.int64):
        a, i = oracle.tokenize(np.array([5, 4, 5, 1, 1], dt))
        assert a.tolist() == [5, 4, 1] and i.tolist() == [0, 1, 0, 2, 2] and i.dtype == np.uint8
    for dt in (np.uint8, np.uint16, np.uint32, np.uint64):
        a, i = oracle.tokenize(np.array([5, 4, 5, 1, 1], dt), sorted_alphabet=True)
        assert a.tolist() == [1, 4, 5] and i.tolist() == [2, 1, 2, 0, 0]
    data = np.arange(300, dtype=np.int32)
    for srt in (False, True):
        a, i = oracle.tokenize(data, sorted_alphabet=srt)
        assert a.tolist() == data.tolist() and i.dtype == np.uint16 and i.tolist() == list(range(300))
