"""The index scheme of the triply periodic fused z kernel (k_tp_zfused),
restated on the CPU: nz = R1 R2, n = R2 n1 + n2, k = k1 + R1 k2; pass 1 takes
DFT_R1 over n1 and the twiddle W^(n2 k1), pass 2 DFT_R2 over n2, each thread
writing back the slots it read, so slot R2 k1 + k2 ends holding X[k1 + R1 k2];
the inverse runs the passes in reverse.  Checked against numpy's FFT for the
sizes the kernel takes, with the radix-2 small DFT and the table-free W_8
twiddles it uses."""
import numpy as np
import pytest

C = 0.70710678118654752440


def _bitrev(i, n):
    r, b = 0, 1
    while b < n:
        r = (r << 1) | (1 if i & b else 0)
        b <<= 1
    return r


def _mul_w8(b, e, inv):
    x, y = b.real, b.imag
    if e == 0:
        return b
    if e == 2:
        return complex(-y, x) if inv else complex(y, -x)
    if e == 1:
        return complex(C * (x - y), C * (x + y)) if inv else complex(C * (x + y), C * (y - x))
    return complex(-C * (x + y), C * (x - y)) if inv else complex(C * (y - x), -C * (x + y))


def _dft_small(v, inv):
    n = len(v)
    u = [v[_bitrev(i, n)] for i in range(n)]
    ln = 2
    while ln <= n:
        for i in range(0, n, ln):
            for k in range(ln // 2):
                b = _mul_w8(u[i + k + ln // 2], k * (8 // ln), inv)
                a = u[i + k]
                u[i + k], u[i + k + ln // 2] = a + b, a - b
        ln *= 2
    return u


@pytest.mark.parametrize("r1,r2", [(4, 4), (8, 4), (8, 8)])
def test_two_pass_digit_reversed_transform(r1, r2):
    nz = r1 * r2
    tw = np.exp(-2j * np.pi * np.arange(nz) / nz)
    rng = np.random.default_rng(nz)
    x = rng.standard_normal(nz) + 1j * rng.standard_normal(nz)
    s = list(x)
    for j in range(r2):  # pass 1, thread n2 = j
        v = _dft_small([s[r2 * n1 + j] for n1 in range(r1)], False)
        for k1 in range(r1):
            s[r2 * k1 + j] = v[k1] * (tw[(j * k1) % nz] if k1 else 1)
    for j in range(r1):  # pass 2, thread k1 = j
        v = _dft_small([s[r2 * j + n2] for n2 in range(r2)], False)
        for k2 in range(r2):
            s[r2 * j + k2] = v[k2]
    X = np.fft.fft(x)
    slots = np.arange(nz)
    assert np.allclose(np.array(s), X[slots // r2 + r1 * (slots % r2)], rtol=0, atol=1e-12)
    for j in range(r1):  # inverse of pass 2
        v = _dft_small([s[r2 * j + k2] for k2 in range(r2)], True)
        for n2 in range(r2):
            s[r2 * j + n2] = v[n2]
    for j in range(r2):  # inverse of pass 1
        v = _dft_small([s[r2 * k1 + j] * (np.conj(tw[(j * k1) % nz]) if k1 else 1) for k1 in range(r1)], True)
        for n1 in range(r1):
            s[r2 * n1 + j] = v[n1]
    assert np.allclose(np.array(s) / nz, x, rtol=0, atol=1e-13)
