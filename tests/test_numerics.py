"""CPU checks of the numerical identities and bounds the sweep kernels rely
on, restated in numpy with the device's operation order and precision.

- the closed form of the Levy bridge (bridge_w): p_t = e + (m-t) (u_0 + sum
  of w_r z_r over r <= t) equals the recursion p_t = a_t p_(t-1) + (1 - a_t)
  e + sigma_t z_t of src/updates/helper.jl:118-139 (the reference's levy!);
- the mirror words formed in FP32 (qcoord) stay within 0.516 units of the
  exact scaled position, the margin the prefilter and estimate bounds take;
- the pair estimates' square-root-free error bounds (EstConst) cover each
  term's error wherever the term is not negligible.
"""
import numpy as np
import pytest

f32 = np.float32


def levy_recursion(s, e, z, lam, tau):
    m = len(z) + 1
    p, out = s, [s]
    for t in range(1, m):
        a = (m - t) / (m + 1 - t)
        sig = np.sqrt(2.0 * lam * a * tau)
        p = a * p + (1.0 - a) * e + z[t - 1] * sig
        out.append(p)
    return np.array(out)


def levy_closed_form(s, e, z, lam, tau):
    m = len(z) + 1
    u, out = (s - e) * (1.0 / m), [s]
    for t in range(1, m):
        a = (m - t) / (m + 1 - t)
        w = np.sqrt(2.0 * lam * a * tau) / (m - t)
        u = u + z[t - 1] * w
        out.append(e + (m - t) * u)
    return np.array(out)


@pytest.mark.parametrize("m", [2, 3, 8, 16, 32, 64])
def test_closed_form_bridge_equals_recursion(m):
    rng = np.random.default_rng(m)
    for _ in range(50):
        s, e = rng.uniform(-8, 8, size=2)
        z = rng.standard_normal(m - 1)
        lam, tau = 0.5, rng.uniform(0.005, 0.1)
        a, b = levy_recursion(s, e, z, lam, tau), levy_closed_form(s, e, z, lam, tau)
        np.testing.assert_allclose(b, a, rtol=0, atol=1e-12 * (1 + np.abs(a).max()))


@pytest.mark.parametrize("L", [5.0, 8.0, 10.0, 16.0, 0.75])
def test_fp32_mirror_words_within_margin(L):
    rng = np.random.default_rng(int(L * 100))
    x = np.concatenate([rng.uniform(-L, L, 200000), np.nextafter(L, 0) * np.array([1.0, -1.0]),
                        np.array([-L, 0.0])])
    scale = 65536.0 / (2.0 * L)
    v = (f32(x) + f32(L)) * f32(scale)           # FP32 sum and product, as qcoord
    word = np.rint(v.astype(np.float64)).astype(np.int64) & 0xFFFF
    exact = (x + L) * scale
    d = (word - exact + 32768.0) % 65536.0 - 32768.0  # wrapped difference in units
    assert np.abs(d).max() <= 0.516


def test_estimate_bounds_cover_the_per_term_errors():
    """a term exp(-y) whose end lies at squared mirror distance d2 has y off
    by at most dy = u^2/(2 s^2) kQErr (2 sqrt(d2) + kQErr) (kQErr = 3 units
    of mirror error on a distance), so its relative error is at most
    exp(dy) - 1 plus __expf's (3 + 1.2 y) ulp.  The device's bounds, formed in
    FP32 as EstConst does (a constant for the first end, which lies within
    q_lim_hi; 2 sqrt(d2) <= d2/s + s for the second), must cover that
    wherever the term is not negligible, and they stay close to the per-term
    bounds they replaced"""
    # C4's chains: L = 8, sigma = 0.5, cell 1.6 (nbins = 10)
    L, sigma, rc = 8.0, 0.5, 1.6
    u = 2.0 * L / 65536.0
    q_u2i = f32(u * u / (2.0 * sigma * sigma))
    rq, e = rc / u, 3.0
    lim_hi = int(np.ceil((rq + e) ** 2))
    kq = f32(3.0)
    c1 = f32(1.01) * q_u2i * kq
    s = np.sqrt(f32(lim_hi), dtype=f32)
    inv_s = f32(1.0) / s
    eps_a = c1 * (f32(2.0) * s + kq) + (f32(3.0) + f32(1.2) * (f32(lim_hi) * q_u2i)) * f32(1.2e-7)

    def required(d2):
        d2 = d2.astype(np.float64)
        y = d2 * float(q_u2i)
        dy = float(q_u2i) * 3.0 * (2.0 * np.sqrt(d2) + 3.0)
        return np.expm1(dy) + (3.0 + 1.2 * y) * 2.0 ** -23

    d2a = np.unique(np.concatenate([np.arange(0, 4096), np.linspace(0, lim_hi, 200001).astype(np.int64)]))
    assert (float(eps_a) >= required(d2a)).all()
    # the second end anywhere the term exp(-y) is above exp(-60)
    d2b = np.unique(np.concatenate([d2a, np.linspace(0, 60.0 / float(q_u2i), 200001).astype(np.int64)]))
    yb = d2b.astype(f32) * q_u2i
    amgm = c1 * (d2b.astype(f32) * inv_s + (s + kq)) + (f32(3.0) + f32(1.2) * yb) * f32(1.2e-7)
    assert (amgm.astype(np.float64) >= required(d2b)).all()
    # within the prefilter reach the second end's bound is at most twice the
    # first end's constant
    near = d2b <= lim_hi
    assert amgm[near].max() <= 2.0 * eps_a
