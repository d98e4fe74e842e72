"""Oracle and CUDA path against fixtures produced by the reference's own code.

The fixtures under tests/golden/ were written by tests/golden/make_golden.py,
which runs the reference sources (GPU kernel on CPU fibers, lookupTable5,
mapHits6, the I/O functions and printOutput).  The oracle is checked against
them on the CPU; the GPU path is checked against them on the GPU.
"""
import json
import os

import pytest

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name, mode="r"):
    with open(os.path.join(G, name), mode) as f:
        return json.load(f) if name.endswith(".json") else f.read()


def b(s: str) -> bytes:
    return s.encode("latin-1")


def test_oracle_sw_pairs(oracle):
    for c in load("sw_pairs.json"):
        got = oracle.sw(b(c["q"]), b(c["w"]), c["Q"], c["R"])
        assert (got["score"], got["start"], got["end"], got["len"]) == (
            c["score"], c["start"], c["end"], c["len"]), c
        assert got["qcons"] == b(c["qcons"]) and got["rcons"] == b(c["rcons"])


def test_oracle_index(oracle):
    g = load("index_k8.json")
    ix = oracle.Index(g["fasta"].encode(), g["k"], g["thres"])
    ri, rp = ix.postings()
    assert list(ri) == g["ref_idx"] and list(rp) == g["ref_pos"]
    for h, start, rep in g["buckets"]:
        assert ix.start(h) == start and ix.repeats(h) == rep


def test_oracle_pipeline(oracle):
    meta = load("pipeline_meta.json")
    got = oracle.align(load("pipeline_ref.fa", "rb"), load("pipeline_reads.fa", "rb"),
                       oracle.default_params(device_mem=meta["device_mem"]))
    assert got == load("pipeline_out.txt", "rb")


def test_oracle_pipeline_sam(oracle):
    # the reference's printOutputSam records of the same inputs
    meta = load("pipeline_meta.json")
    got = oracle.align(load("pipeline_ref.fa", "rb"), load("pipeline_reads.fa", "rb"),
                       oracle.default_params(device_mem=meta["device_mem"], out_format=1))
    assert got == load("pipeline_out_sam.txt", "rb")


def test_oracle_pipeline_lt13(oracle):
    # the reference's lookupTable13 kernel (run on CPU fibers) made this file
    meta = load("pipeline_meta.json")
    got = oracle.align(load("pipeline_ref.fa", "rb"), load("pipeline_reads.fa", "rb"),
                       oracle.default_params(device_mem=meta["device_mem"], seeder=1))
    assert got == load("pipeline_out_lt13.txt", "rb")


@pytest.mark.gpu
def test_gpu_pipeline_lt13():
    import swift_gb300 as sg
    meta = load("pipeline_meta.json")
    ctx = sg.Context(0)
    ix = ctx.index(load("pipeline_ref.fa", "rb"))
    got = ctx.align(ix, load("pipeline_reads.fa", "rb"),
                    sg.default_params(device_mem=meta["device_mem"], seeder=1))
    assert got == load("pipeline_out_lt13.txt", "rb")


@pytest.mark.gpu
def test_gpu_pipeline_sam():
    import swift_gb300 as sg
    meta = load("pipeline_meta.json")
    ctx = sg.Context(0)
    ix = ctx.index(load("pipeline_ref.fa", "rb"))
    want = load("pipeline_out_sam.txt", "rb")
    for dm in (meta["device_mem"], 100_000_000 + 24 * 1220):  # one batch; batches of 24
        got = ctx.align(ix, load("pipeline_reads.fa", "rb"),
                        sg.default_params(device_mem=dm, out_format=1))
        assert got == want


@pytest.mark.gpu
def test_gpu_sw_pairs():
    import swift_gb300 as sg
    ctx = sg.Context(0)
    cases = load("sw_pairs.json")
    by_dims = {}
    for c in cases:
        by_dims.setdefault((c["Q"], c["R"]), []).append(c)
    for (Q, R), cs in by_dims.items():
        got = ctx.sw_batch([b(c["q"]) for c in cs], [b(c["w"]) for c in cs], Q, R)
        for g, c in zip(got, cs):
            assert (g["score"], g["start"], g["end"], g["len"], g["qcons"], g["rcons"]) == (
                c["score"], c["start"], c["end"], c["len"], b(c["qcons"]), b(c["rcons"])), c


@pytest.mark.gpu
def test_gpu_index():
    import swift_gb300 as sg
    g = load("index_k8.json")
    ctx = sg.Context(0)
    look, rep, ri, rp = ctx.index(g["fasta"].encode(), g["k"], g["thres"]).export()
    assert list(ri) == g["ref_idx"] and list(rp) == g["ref_pos"]
    for h, start, r in g["buckets"]:
        assert look[h] == start and rep[h] == r


@pytest.mark.gpu
def test_gpu_pipeline():
    import swift_gb300 as sg
    meta = load("pipeline_meta.json")
    ctx = sg.Context(0)
    ix = ctx.index(load("pipeline_ref.fa", "rb"))
    got = ctx.align(ix, load("pipeline_reads.fa", "rb"),
                    sg.default_params(device_mem=meta["device_mem"]))
    assert got == load("pipeline_out.txt", "rb")
