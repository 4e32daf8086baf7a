"""The planner's default schedules (no GPU: plans are built on the host).

The rules were set from gl_plan_autotune measurements on GB300; these tests
pin them so that a change to the planner shows up here:
  * two passes with a 512-point first pass for 2^16 .. 2^21 and the mixed
    lengths near 2^20, a 64-point first pass up to 2^15, four-lane kernels;
  * the split nearest sqrt(n) above (2^22 .. 2^24, 16 711 680) and where the
    short-first-pass rule would need the run-time-radix kernel;
  * three passes: a 512-point first pass, a middle pass nearest 64 points,
    the largest compiled last pass."""
import pytest


def gpu(gl, n):
    return gl.strategy(n).describe().split(" | gpu: ")[1]


@pytest.fixture(autouse=True)
def _defaults(gl):
    from goldilocks_gb300 import tune
    tune.clear()
    yield
    tune.clear()


@pytest.mark.parametrize("n,want", [
    (1 << 12, "col 64 (8x8x1, 4 lanes) + row 64 (8x8x1, 4 lanes)"),
    (1 << 13, "col 64 (8x8x1, 4 lanes) + row 128 (16x8x1, 4 lanes)"),
    (1 << 15, "col 64 (8x8x1, 4 lanes) + row 512 (8x8x8, 4 lanes)"),
    (1 << 16, "col 512 (8x8x8, 4 lanes) + row 128 (16x8x1, 4 lanes)"),
    (1 << 18, "col 512 (8x8x8, 4 lanes) + row 512 (8x8x8, 4 lanes)"),
    (1 << 20, "col 512 (8x8x8, 4 lanes) + row 2048 (16x16x8, 4 lanes)"),
    (1 << 21, "col 512 (8x8x8, 4 lanes) + row 4096 (16x16x16, 4 lanes)"),
    (5 << 18, "col 512 (8x8x8, 4 lanes) + row 2560 (16x16x10, 4 lanes)"),
    (17 << 16, "col 512 (8x8x8, 4 lanes) + row 2176 (16x8x17, 4 lanes)"),
    (1 << 22, "col 2048 (16x16x8, 2 lanes) + row 2048 (16x16x8, 2 lanes)"),
    (1 << 24, "col 4096 (16x16x16, 4 lanes) + row 4096 (16x16x16, 4 lanes)"),
    (16711680, "col 4096 (16x16x16, 4 lanes) + row 4080 (16x15x17, 4 lanes, Good-Thomas)"),
    (15 << 20, "col 4096 (16x16x16, 4 lanes) + row 3840 (16x16x15, 4 lanes)"),
])
def test_two_pass_defaults(gl, n, want):
    assert gpu(gl, n) == want


def test_short_first_pass_needs_compiled_passes(gl):
    # 6144 = 64 x 96 would put 96 points on the run-time-radix kernel: the
    # split nearest sqrt(n) is kept.
    assert not gpu(gl, 6144).startswith("col 64 ")


@pytest.mark.parametrize("n,want", [
    (1 << 25, "col 512 (8x8x8, 4 lanes) + col 64 (8x8x1, 4 lanes) + row 1024 (16x8x8, 2 lanes)"),
    (1 << 28, "col 512 (8x8x8, 4 lanes) + col 128 (16x8x1, 4 lanes) + row 4096 (16x16x16, 4 lanes)"),
    (3 << 24, "col 512 (8x8x8, 4 lanes) + col 64 (8x8x1, 4 lanes) + row 1536 (16x16x6, 4 lanes)"),
    (17 << 21, "col 512 (8x8x8, 4 lanes) + col 64 (8x8x1, 4 lanes) + row 1088 (16x4x17, 4 lanes)"),
    (255 << 17, "col 256 (16x16x1, 4 lanes) + col 64 (8x8x1, 4 lanes) + row 2040 (8x15x17, 4 lanes)"),
])
def test_three_pass_defaults(gl, n, want):
    assert gpu(gl, n) == want


def test_no_compiled_shape_left_unused(gl):
    """Every length up to 2^24 whose split reaches a pass size with a compiled
    kernel uses it: the run-time-radix kernel only appears for pass sizes that
    have none (the two are labelled apart)."""
    compiled = {"1536", "2560", "3072", "3840", "1280", "1920", "4080", "2176", "2040",
                "2720", "3264", "1360", "1632", "1088", "768", "640", "480", "384", "320",
                "272", "544", "680", "408", "340"}
    for n in gl.divisors():
        if n <= 4096 or n > 1 << 24 or n % 257 == 0 or n % 65537 == 0:
            continue
        for part in gpu(gl, n).split(" + "):
            size = part.split()[1]
            if size in compiled:
                assert "run-time radices" not in part, (n, part)


def test_no_run_time_radix_pass_from_2p16_to_2p24(gl):
    for n in gl.divisors():
        if n < 1 << 16 or n > 1 << 24 or n % 257 == 0 or n % 65537 == 0:
            continue
        assert "run-time radices" not in gpu(gl, n), (n, gpu(gl, n))
