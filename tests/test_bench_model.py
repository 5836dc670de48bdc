"""bench.py's byte models (the roofline denominators' numerators): the per-operator and per-solve
figures of the headline workload, and the per-stage bytes summing to the pipeline's traffic."""
import importlib.util
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_models", os.path.join(ROOT, "bench.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_headline_byte_model():
    b = _bench()
    per_op = b.normal_op_model_bytes(32, 256, 512, 16384)
    assert abs(per_op - 580.1e6) < 0.1e6            # 580.1 MB per 32-coil normal operator
    assert abs(b.SOLVE_MODEL_BYTES - 18.27e9) < 0.01e9   # 1 adjoint + 31 normal operators


def test_stage_bytes_of_the_pipeline():
    b = _bench()
    cc, N, G = 32, 256, 512
    st = b.stage_bytes(cc, N, G, 16384, 4, False)
    assert len(st) == 5
    img, grid, half = N * N * 8, G * G * 8, G * N * 8
    assert st[2] == 2 * cc * grid                      # gridding: grid in + grid out
    assert st[1] == st[3] == cc * half + cc * grid     # the two strided/contiguous middle passes
    assert abs(sum(st) - 471.3e6) < 0.1e6              # what the 32-coil pipeline moves
    sten = b.stage_bytes(cc, N, G, 16384, 4, True)
    assert sten[2] - st[2] == 49 * G * G * 4            # + the (2W-1)^2 stencil weights once
