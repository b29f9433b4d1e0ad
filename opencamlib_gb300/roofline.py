"""Frozen work figures of the drop-cutter kernels, for the compute roofline.

The drop path is bound by FP32 issue (the screen) and FP64 issue (the
refinement, the bull's edge solves, handed-back points), not by HBM.  Its
unit of work is one (CL point, triangle) pair: the library counts the pairs
the FP32 screen evaluated (`screened`) and the triangles the FP64 stages
evaluated (`refined`) in every call's statistics.  The figures below turn
those counts into floating-point operations:

  FP32_PER_SCREEN[c]   FP32 operations (add, mul = 1, fused multiply-add = 2)
                       executed by all screen kernels of cutter c, per
                       screened pair;
  FP64_PER_REFINED[c]  FP64 operations executed by all FP64 kernels of the
                       call (refinement, bull edge solves, handed-back
                       points), per refined triangle.

They are the ncu instruction counters (smsp__sass_thread_inst_executed_op_
{fadd,fmul,ffma,dadd,dmul,dfma}_pred_on.sum) summed over the kernels of one
call on the 256 x 256-point block of the benchmark raster, divided by that
call's own counters (the capture and the arithmetic are kept with the ncu
summaries under profiles/).  A step's roofline time is then

  T_roof = sum_c screened_c * FP32_PER_SCREEN[c] / P32
         + sum_c refined_c  * FP64_PER_REFINED[c] / P64

with P32, P64 the FMA throughput measured on the device
(ocl_gb300_fma_peaks), and the fraction is T_roof / T_step.

SCREEN_DRAM_BYTES[c] is the DRAM traffic (dram__bytes_read.sum +
dram__bytes_write.sum) of the screen kernels (seeding, dense and sparse
screen) of one call on the full 1,000,000-point raster, from a one-pass
ncu capture of `bench.py --profile-step` (summarised under profiles/).
"""
from __future__ import annotations

# cutter -> FP32 operations per screened pair
FP32_PER_SCREEN = {"cyl": 565.2, "ball": 694.0, "bull": 1214.0, "cone": 748.6, "ballcone": 1567.1}
# cutter -> FP64 operations per refined triangle
FP64_PER_REFINED = {"cyl": 129.5, "ball": 256.8, "bull": 1274.3, "cone": 295.6, "ballcone": 320.6}
# cutter -> DRAM bytes of the screen kernels per call on the 1,000,000-point raster
SCREEN_DRAM_BYTES = {"cyl": 784473344, "ball": 688323584, "bull": 854738432, "cone": 547958272, "ballcone": 959312384}


def measured(names) -> bool:
    return all(FP32_PER_SCREEN.get(n) is not None and FP64_PER_REFINED.get(n) is not None for n in names)


def step_roofline(per_cutter_counts, step_seconds, p32_flops, p64_flops):
    """per_cutter_counts: {cutter: (screened, refined)} of one step.
    Returns a dict with the step's FP32 and FP64 operations, the roofline
    time and its fraction of the measured step time; the FP64 operations are
    also given as FP32-equivalent work (times P32 / P64) so the step has one
    achieved rate against the FP32 peak."""
    f32 = sum(s * FP32_PER_SCREEN[c] for c, (s, r) in per_cutter_counts.items())
    f64 = sum(r * FP64_PER_REFINED[c] for c, (s, r) in per_cutter_counts.items())
    t_roof = f32 / p32_flops + f64 / p64_flops
    equiv = f32 + f64 * (p32_flops / p64_flops)
    return {"fp32_ops": f32, "fp64_ops": f64, "t_roof_s": t_roof, "t_step_s": step_seconds,
            "achieved_flops_fp32_equiv": equiv / step_seconds, "frac": t_roof / step_seconds}
