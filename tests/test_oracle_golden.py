"""The CPU restatement against the reference's own known-answer tests.

Every case below is an input and expected result written in the reference's
unit tests (file:line cited per case).  Where the reference accepts any
member of a tie set, the deterministic rule of the restatement (first in
sort order) must pick a member of that set.
"""
import pytest

# --- test/testSmithWaterman.cu ------------------------------------------


def test_sw_kernel_full(oracle):
    # test/testSmithWaterman.cu:29-124 (smithWaterman kernel)
    r = oracle.sw(b"ACGTACGTAA", b"CCCCAAAACGTCCGTTACGT")
    assert r["score"] == 14.0
    assert (r["start"], r["end"], r["len"]) == (8, 17, 10)
    assert r["qcons"] == b"AATGCATGCA"
    assert r["rcons"] == b"ATTGCCTGCA"


def _bit(dirs, R, byte, bit):
    """Cell index of bit `bit` (LSB=0) of byte `byte` of the reference's
    MSB-first bit planes (src/smithWaterman.cu:575-611)."""
    cell = byte * 8 + (7 - bit)
    return dirs.reshape(-1)[cell]


def test_sw_compute_max_score_no_gaps(oracle):
    # test/testSmithWaterman.cu:130-214
    r = oracle.sw(b"ACGTACGTAA", b"CCCCAAAACGTCCGTTACGT", want_dirs=True)
    assert r["score"] == 14.0 and r["cell_max"] == 227
    d = r["dirs"]
    for byte, bit in [(3, 2), (6, 4), (9, 6), (11, 0), (14, 2), (17, 4), (20, 6),
                      (22, 0), (25, 2), (28, 4)]:
        assert _bit(d, 20, byte, bit) not in (2, 3)  # neither UP nor LEFT


def test_sw_compute_max_score_gaps(oracle):
    # test/testSmithWaterman.cu:216-301
    r = oracle.sw(b"CTTGTCACCATCCA", b"CTTGTCACCATCA", want_dirs=True)
    assert r["score"] == 24.0 and r["cell_max"] == 180
    d = r["dirs"]
    for byte, bit in [(1, 0), (3, 1), (5, 2), (7, 3), (9, 4), (11, 5), (13, 6),
                      (15, 7), (16, 0), (18, 1), (20, 2), (22, 3)]:
        assert _bit(d, 13, byte, bit) not in (2, 3)


def test_sw_compute_max_score_short_reference(oracle):
    # test/testSmithWaterman.cu:304-386: refLen 25 > 20 bases present
    r = oracle.sw(b"ACGTACGTAA", b"CCCCAAAACGTCCGTTACGT", R=25)
    assert r["score"] == 14.0 and r["cell_max"] == 277


def test_sw_backtrack(oracle):
    # test/testSmithWaterman.cu:394-514
    r = oracle.sw(b"ACGTACGTAA", b"CCCCAAAACGTCCGTTACGT")
    assert (r["score"], r["start"], r["end"], r["len"]) == (14.0, 8, 17, 10)
    assert r["qcons"] == b"AATGCATGCA" and r["rcons"] == b"ATTGCCTGCA"


# --- test/testMapHits6.cu -----------------------------------------------

def test_best_hits_one(oracle):
    # test/testMapHits6.cu:199-226
    got = oracle.best_hits(3, [1, 2, 2], [5, -1, -1], [20, 10, 30])
    assert got == [(2, -1, 10)]


def test_best_hits_two(oracle):
    # test/testMapHits6.cu:228-260
    got = oracle.best_hits(3, [1, 2, 2, 3, 3], [5, -1, -1, 5, 5], [20, 10, 30, 30, 40])
    assert got == [(2, -1, 10), (3, 5, 30)]


def test_best_hits_tie_limited(oracle):
    # test/testMapHits6.cu:262-291: either biggest cluster is accepted
    got = oracle.best_hits(1, [1, 2, 2, 3, 3], [5, -1, -1, 5, 5], [20, 10, 30, 30, 40])
    assert len(got) == 1 and got[0] in [(2, -1, 10), (3, 5, 30)]


def test_best_hits_empty(oracle):
    # src/mapHits6.cu:46-47
    assert oracle.best_hits(3, [], [], []) == []


# --- test/testLookupTable5.cu -------------------------------------------

def test_index_one_reference(oracle):
    # test/testLookupTable5.cu:33-68
    ix = oracle.Index(b">ref1\nACGTACGTGTACGTAACATC\n", k=8, thres=15)
    assert ix.num_buckets == 65536
    assert ix.start(3662) == 1 and ix.start(58596) == 2
    ri, rp = ix.postings()
    assert list(ri) == [-1, 0, 0] and list(rp) == [-1, 8, 0]
    assert ix.repeats(3662) == 1 and ix.repeats(58596) == 1


THREE_REF_STARTS = {3648: 1, 3662: 2, 14649: 3, 17636: 5, 20032: 6, 37056: 7,
                    37782: 8, 58416: 9, 58596: 10, 58597: 12, 58599: 13, 64740: 14}
THREE_REF_IDX = [-1, 1, 2, 2, 1, 0, 2, 2, 1, 0, 1, 0, 0, 2, 0]
THREE_REF_POS = [-1, 16, 32, 0, 24, 24, 24, 8, 0, 8, 8, 0, 32, 16, 16]
THREE_REF_REPEATS = {3648: 1, 3662: 1, 14649: 2, 17636: 1, 20032: 1, 37056: 1,
                     37782: 1, 58416: 1, 58596: 2, 58597: 1, 58599: 1, 64740: 1}


@pytest.mark.parametrize("fasta,thres", [
    # test/testLookupTable5.cu:71-160: one line per reference
    (b">ref1\nACGTACGTAATAACGTACGTATTTACGTACACCCGTACGT\n>ref2\n"
     b"GCCGTACGACGTACGTAAACGTAACGTACGTATTTACG\n"
     b">ref3\nCGTACGTAAAATAACGTCGTACGTAAACGTACGTACGTAA", 15),
    # test/testLookupTable5.cu:163-253: sequences split over lines, T=4
    (b">ref1\nACGTACGTAATAACGTACGTATTT\nACGTACACCCGTACGT\n>ref2\n"
     b"GCCGTACGACGTACGTAAACGTAA\nCGTACGTATTTACG\n"
     b">ref3\nCGTACGTAAA\nATAACGTCGT\nACGTAAACGT\nACGTACGTAA", 4),
])
def test_index_three_references(oracle, fasta, thres):
    ix = oracle.Index(fasta, k=8, thres=thres)
    for h, s in THREE_REF_STARTS.items():
        assert ix.start(h) == s
    ri, rp = ix.postings()
    assert list(ri) == THREE_REF_IDX
    assert list(rp) == THREE_REF_POS
    for h, c in THREE_REF_REPEATS.items():
        assert ix.repeats(h) == c


def test_index_ignore_threshold(oracle):
    # test/testLookupTable5.cu:256-350: k=4, T=7, one tuple over threshold
    fasta = (b">ref1\nACGTACGTAATAACGTACGTATTT\nACGTACACCCGTACGT\n>ref2\n"
             b"GCCGTACGACGTACGTAAACGTAA\nCGTACGTATTTACG\n"
             b">ref3\nCGTACGTAAA\nATAACGTCGT\nACGTAAACGT\nACGTACGTAA")
    ix = oracle.Index(fasta, k=4, thres=7)
    assert ix.num_buckets == 256
    starts = {14: 1, 48: 3, 57: 4, 63: 8, 64: 9, 68: 11, 78: 12, 144: 14, 147: 15,
              150: 16, 192: 17, 229: 18, 231: 19, 252: 20}
    for h, s in starts.items():
        assert ix.start(h) == s
    ri, rp = ix.postings()
    assert list(ri) == [-1, 2, 1, 0, 2, 2, 1, 1, 1, 2, 1, 0, 2, 2, 2, 1, 1, 2, 0, 2, 0]
    assert list(rp) == [-1, 36, 20, 8, 4, 0, 28, 24, 32, 24, 16, 28, 32, 28, 12, 4, 0,
                        8, 32, 16, 20]
    reps = {14: 2, 48: 1, 57: 4, 63: 1, 64: 2, 68: 1, 78: 2, 144: 1, 147: 1, 150: 1,
            192: 1, 229: 1, 231: 1, 252: 1}
    for h, c in reps.items():
        assert ix.repeats(h) == c


def test_map_query_one_reference(oracle):
    # test/testLookupTable5.cu:355-394 (maxNumHits 10)
    ix = oracle.Index(b">ref1\nACGTACGTGTACGTAACATC\n", k=8, thres=15)
    assert ix.map_query(b"ACGTACGTAA", 10) == [(0, 0, 0), (0, 6, 8)]
    assert ix.map_query(b"TTACGTACGT", 10) == [(0, -2, 0)]


THREE_REF_1LINE = (b">ref1\nACGTACGTACGTACGTACGT\n>ref2\nGCCGTACGACGTACGT\n"
                   b">ref3\nCGTACGTAAAATAA")


def test_map_query_three_references(oracle):
    # test/testLookupTable5.cu:397-485: any two of the tied clusters
    ix = oracle.Index(THREE_REF_1LINE, k=8, thres=15)
    fwd = ix.map_query(b"ACGTACGTAA", 2)
    allowed = {(0, 0, 0), (0, 8, 8), (1, 8, 8), (2, -1, 0)}
    assert len(fwd) == 2 and set(fwd) <= allowed
    assert fwd == [(0, 0, 0), (0, 8, 8)]  # first two in sort order
    rev = ix.map_query(b"TTACGTACGT", 2)
    allowed = {(0, -2, 0), (0, 6, 8), (1, 6, 8)}
    assert len(rev) == 2 and set(rev) <= allowed


# --- test/testQuery.cu ----------------------------------------------------

def test_revcomp(oracle):
    # src/query.cu:265-282: A<->T, C<->G, anything else -> A
    assert oracle.revcomp(b"ACGTACGTAA") == b"TTACGTACGT"
    assert oracle.revcomp(b"ACGTN") == b"AACGT"
    assert oracle.revcomp(b"acgt") == b"AAAA"


def test_hash(oracle):
    # src/preprocess.cu:70-91: base-4 little-endian, N and others -> A
    assert oracle.hash_kmer(b"ACG", 3) == 36
    assert oracle.hash_kmer(b"acg", 3) == 36
    assert oracle.hash_kmer(b"NNN", 3) == 0
    assert oracle.hash_kmer(b"TTTT", 4) == 255
