"""Register spills of the sm_103a kernels, from the ptxas reports the build keeps (CPU).

The hot kernels -- the single-grid fused stage kernels (FP64 fixed-point and taps,
FP32), the decomposed stage kernel, the batched advection kernel, the line, 3D ring
and tensor-core convolution kernels -- must not spill. Three families have a measured
ceiling instead:
- wave_batch_fixed_kernel: 14 compute, 6 converter and 1 producer warp per CTA; with
  21 warps one SM sub-partition holds 6 of them, so its 16,384 registers allow 80 a
  thread, and the order-2/4/6 tiles spill up to 60 bytes at that ceiling;
- wave3d_stage_kernel: the 3D column kernel, the fallback for states the ring kernel
  cannot take (unaligned pointers, planes of 2^31 elements), capped by its occupancy
  bounds;
- wave_batch_stage_kernel: 8 bytes in the FP32 order-6 entries with 96 registers.
A kernel that starts to spill, or a family that spills more, fails here."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# family -> (spill-store ceiling, spill-load ceiling) in bytes; every other kernel: (0, 0)
CEILINGS = {
    "wave_batch_fixed_kernel": (64, 96),
    "wave3d_stage_kernel": (176, 160),
    "wave_batch_stage_kernel": (8, 8),
}
HOT = ["wave_fixed_kernel", "wave_stage_kernel", "adv_batch_stage_kernel", "wave_batch_stage_kernel",
       "wave_batch_fixed_kernel", "line_stage_kernel", "wave3d_ring_kernel", "conv3x3_tc_kernel",
       "conv3x3_wgrad_tc_kernel", "hnorm_partial_kernel", "error_partial_kernel"]


def _family(mangled: str):
    """The kernel name of a mangled symbol: the first length-prefixed identifier after sbp's
    namespace (Itanium mangling: N3sbp<len><name>, or 3sbp<len>... for function templates)."""
    for name in HOT + list(CEILINGS):
        if f"{len(name)}{name}" in mangled:
            return name
    return None


@pytest.fixture(scope="module")
def report():
    sys.path.insert(0, os.path.join(ROOT, "hpc-reading-course_gb300"))
    import build as gpu_build

    gpu_build.build()
    try:
        return gpu_build.resource_report()
    except FileNotFoundError:  # built before the reports were kept
        gpu_build.build(force=True)
        return gpu_build.resource_report()


def test_every_hot_kernel_is_reported(report):
    families = {_family(k) for k in report}
    for name in HOT:
        assert name in families, name


@pytest.mark.parametrize("family", [None] + HOT, ids=["other"] + HOT)
def test_no_spills_beyond_the_measured_ceilings(report, family):
    st_max, ld_max = CEILINGS.get(family, (0, 0))
    bad = [(k, r["spill_stores"], r["spill_loads"]) for k, r in report.items()
           if _family(k) == family and (r["spill_stores"] > st_max or r["spill_loads"] > ld_max)]
    assert not bad, bad


def test_registers_within_the_file(report):
    """No kernel asks for more than the 255 registers a thread can address."""
    assert all(0 < r["registers"] <= 255 for r in report.values())
