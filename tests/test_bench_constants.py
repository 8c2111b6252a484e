"""The bench's frozen per-pair instruction counts belong to one version of the kernel sources.

bench.py turns the df64 M_UF kernel's CUDA-event time into a fraction of the FP32 issue peak with an
instruction count per ordered pair taken from an ncu capture.  That constant is only valid for the
kernel it was measured on: this test fails as soon as the sources that fix the kernel's instruction
stream change, so that a kernel edit cannot silently stale the reported roofline fraction.
"""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_df64_instruction_constants_match_the_kernel_sources():
    import bench
    assert bench.df64_uf_kernel_source_sha() == bench.DF64_UF_KERNEL_SOURCE_SHA, (
        "the df64 M_UF kernel sources changed: capture smsp__inst_executed.sum and the DRAM bytes of the "
        "symmetric and one-sided kernels again and update DF64_UF_INST_PER_PAIR, DF64_UF_TRAFFIC_BYTES and "
        "DF64_UF_KERNEL_SOURCE_SHA in bench.py (and the profile summary)")


def test_roofline_fractions_are_consistent():
    import bench
    ipp = bench.DF64_UF_INST_PER_PAIR
    assert 300 < ipp["symmetric"] < ipp["standard"] < 1000
    assert bench.FLOPS_PER_PAIR == {"uf": 200.0, "ut": 115.0, "wf": 115.0, "wt": 125.0}
