"""Algorithmic work constants of the path tracer, used by the benchmark's
roofline figures (one place, so the numerator of every roofline fraction is
the same count).

Unit of work: one path segment = one trace_ray call (src/renderer/cpu.rs:257).
FP32 operations are counted as in the reference's source, each add, sub, mul,
div, sqrt, min, max and compare as 1 (the reference has no FMA):

  sphere test (cpu.rs:34-62)  ~24 ops   (hoisting d.d, o.d, o.o per ray and
  cube test   (cpu.rs:64-98)  ~24 ops    c.c, r*r, slab bounds per object)
  shading, scatter, RNG mapping, accumulation per segment  ~100 ops

so ops/segment = 24 * objects + 100.  The bound is the FP32 issue rate: SMs x
128 lanes x SM clock, measured in the same run by rdc_measure_fp32_issue
(one lane operation per clock; non-contracted code cannot use the second
operation of an FFMA).
"""

OPS_PER_PRIMITIVE_TEST = 24
OPS_PER_SEGMENT_SHADE = 100


def ops_per_segment(n_objects: int) -> int:
    return OPS_PER_PRIMITIVE_TEST * int(n_objects) + OPS_PER_SEGMENT_SHADE
