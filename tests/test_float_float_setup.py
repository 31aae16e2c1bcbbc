"""The float-float node setup of the mixed path, restated in numpy float32 (CPU only).

The kernels form an interpolation weight (x[k+1] - arg) / (x[k+1] - x[k]) from an argument that is
a sum of the node and task frequencies.  Rounded to FP32, the argument carries |arg| ulps, which
the division by the spacing amplifies up to ~N ulps on an N-point lin-tanh mesh; carried as a pair
h + l of floats (error-free two-sum additions) and subtracted pairwise, the weight keeps the
rounding of the weight itself.  This test restates that arithmetic (make_plan_ff / get_param_ff in
pffrg_device.cuh) and checks both claims on the benchmark meshes.
"""
import numpy as np

f32 = np.float32


def ff(x):
    h = f32(x)
    return (h, f32(x - float(h)))


def ff_add(a, b):
    s = f32(a[0] + b[0])
    bb = f32(s - a[0])
    e = f32(f32(a[0] - f32(s - bb)) + f32(b[0] - bb))
    t = f32(f32(e + a[1]) + b[1])
    h = f32(s + t)
    return (h, f32(t - f32(h - s)))


def weights_ff(val, xs):
    """(lo, hi, wl, wu) of the interval containing the pair val (inside the mesh)."""
    hs = np.array([ff(x)[0] for x in xs])
    ls = np.array([ff(x)[1] for x in xs])
    hi = int(np.searchsorted(hs, val[0], side="left"))
    if hs[hi] == val[0] and ls[hi] < val[1]:
        hi += 1
    lo = hi - 1 if (val[0] < hs[hi] or (val[0] == hs[hi] and val[1] < ls[hi])) else hi
    d = f32(1.0 / (xs[hi] - xs[lo]))
    wl = d * f32(f32(hs[hi] - val[0]) + f32(ls[hi] - val[1]))
    wu = d * f32(f32(val[0] - hs[lo]) + f32(val[1] - ls[lo]))
    return lo, hi, float(wl), float(wu)


def weights_f32(val, xs):
    x32 = xs.astype(f32)
    v = f32(val)
    hi = int(np.searchsorted(x32, v, side="left"))
    lo = hi - 1 if v < x32[hi] else hi
    d = f32(1.0 / (xs[hi] - xs[lo]))
    return lo, hi, float(d * f32(x32[hi] - v)), float(d * f32(v - x32[lo]))


def weights_f64(val, xs):
    hi = int(np.searchsorted(xs, val, side="left"))
    lo = hi - 1 if val < xs[hi] else hi
    d = 1.0 / (xs[hi] - xs[lo])
    return lo, hi, d * (xs[hi] - val), d * (val - xs[lo])


def test_float_float_weights_keep_fp32_rounding_of_the_weight(pkg):
    import pffrg_gb300.workloads as wl

    lat, r, m, a = wl.build_state(wl.WORKLOADS["pyrochlore-L6-2l"])
    rng = np.random.default_rng(0)
    worst = {}
    for name, xs in (("sigma", m.sigma), ("omega", m.omega_s), ("nu", m.nu_s)):
        worst_ff = worst_32 = 0.0
        for _ in range(2000):
            v = rng.uniform(-1.0, 1.0) * xs[-1] * rng.choice([0.01, 0.1, 1.0])
            w = xs[rng.integers(len(xs))]
            val64 = abs(v + 0.5 * w)
            if not (xs[0] < val64 < xs[-1]):
                continue
            val = ff_add(ff(v), (f32(0.5) * ff(w)[0], f32(0.5) * ff(w)[1]))
            if val[0] < 0:
                val = (-val[0], -val[1])
            p64, pff, p32 = weights_f64(val64, xs), weights_ff(val, xs), weights_f32(val64, xs)
            if pff[:2] == p64[:2]:
                worst_ff = max(worst_ff, abs(pff[2] - p64[2]), abs(pff[3] - p64[3]))
            if p32[:2] == p64[:2]:
                worst_32 = max(worst_32, abs(p32[2] - p64[2]), abs(p32[3] - p64[3]))
        assert worst_ff < 2.5e-7  # a couple of FP32 ulps of a weight in [0, 1]
        assert worst_32 >= worst_ff
        worst[name] = (worst_ff, worst_32)
    # on the 51-point σ mesh the plain FP32 weight is off by many ulps
    assert worst["sigma"][1] > 4 * worst["sigma"][0]
