"""The mixed operator's own x-y transforms (dpst_fft.cu) through the C ABI
diagnostic dpst_xy_transform: the forward transform of random FP32 planes
against torch's FP64 rfft2 (max error 2e-6 of the largest coefficient), the
inverse of the forward giving back nx ny times the input (2e-6), and the
inverse of a non-Hermitian spectrum against torch's irfft2 (which, like the
operator, keeps the real-part convention of a complex-to-real transform);
and the mixed operator with its own transforms against the same operator on
cuFFT's (5e-6: two FP32 computations of the same transform).  The
one-launch form (both passes in one persistent kernel, the intermediate in
L2) gives the two-pass results (the same arithmetic per value, 1e-6 of the
largest value allowing for the compiler's contraction choices), on repeated
launches (its counters reset themselves), and the operator with it
matches the two-pass operator, for one right-hand side and for K columns
(more planes than the handle's own grid)."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from conftest import rel_err  # noqa: E402
from doublyperiodicstokes_gb300 import DPStokes, StokesParams, _lib, workloads as W  # noqa: E402

pytestmark = pytest.mark.gpu
SIZES = [(64, 32), (128, 128), (256, 64), (512, 512), (1024, 256), (2048, 1024), (64, 1024), (256, 512), (128, 512)]
FUSED = [(128, 128), (256, 256), (512, 512), (1024, 1024)]
CLUSTER = [(256, 256), (512, 512)]


def _xy(nx, ny, planes, src, dst, inverse, form=0):
    L = _lib.lib()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(L.dpst_xy_transform(nx, ny, planes, ctypes.c_void_p(src.data_ptr()), ctypes.c_void_p(dst.data_ptr()),
                                   int(inverse), int(form), torch.cuda.current_device(), stream))


@pytest.mark.parametrize("nx,ny", SIZES)
def test_forward_and_round_trip(nx, ny):
    planes = 3
    g = torch.Generator(device="cuda").manual_seed(nx + ny)
    x = torch.randn(planes, ny, nx, device="cuda", generator=g, dtype=torch.float32)
    spec = torch.empty(planes, ny, nx // 2 + 1, dtype=torch.complex64, device="cuda")
    _xy(nx, ny, planes, x, spec, False)
    ref = torch.fft.rfft2(x.double())
    err = float((spec.to(torch.complex128) - ref).abs().max() / ref.abs().max())
    print("%d x %d forward max err %.2e" % (nx, ny, err))
    assert err < 2e-6
    back = torch.empty_like(x)
    _xy(nx, ny, planes, spec, back, True)
    err2 = float((back.double() / (nx * ny) - x.double()).abs().max() / x.abs().max())
    print("%d x %d round trip max err %.2e" % (nx, ny, err2))
    assert err2 < 2e-6


@pytest.mark.parametrize("nx,ny", [(128, 64), (512, 512)])
def test_inverse_of_general_spectrum(nx, ny):
    planes = 2
    g = torch.Generator(device="cuda").manual_seed(7)
    s = torch.randn(planes, ny, nx // 2 + 1, 2, device="cuda", generator=g)
    spec = torch.view_as_complex(s.contiguous())
    ref = torch.fft.irfft2(spec.to(torch.complex128), s=(ny, nx)) * (nx * ny)
    out = torch.empty(planes, ny, nx, dtype=torch.float32, device="cuda")
    _xy(nx, ny, planes, spec.clone(), out, True)
    err = float((out.double() - ref).abs().max() / ref.abs().max())
    print("%d x %d inverse max err %.2e" % (nx, ny, err))
    assert err < 2e-6


@pytest.mark.parametrize("name", ["s_dp_t", "c2_dp_n65536@128", "c1_dpsc_n16384", "c0_dpbw_n2048"])
def test_operator_own_fft_matches_cufft(name, monkeypatch):
    w = W.SMALL_BY_NAME.get(name) or W.by_name(name)
    X, F, T = W.make_inputs(w)
    out = {}
    for which in ("own", "cufft"):
        if which == "cufft":
            monkeypatch.setenv("DPSTOKES_GB300_XY_FFT", "cufft")
        op = DPStokes(StokesParams.from_workload(w, "mixed"), w.N)
        own = op.info()["xy_transform"]
        op.set_positions(torch.tensor(X, device=op.device))
        V, Wv = op.mdot(torch.tensor(F, dtype=torch.float32, device=op.device),
                        torch.tensor(T, dtype=torch.float32, device=op.device) if T is not None else None)
        torch.cuda.synchronize()
        out[which] = (own, V.double().cpu().numpy(), Wv.double().cpu().numpy() if Wv is not None else None)
        op.close()
    pow2 = (w.nx & (w.nx - 1)) == 0 and (w.ny & (w.ny - 1)) == 0 and w.nx >= 64 and w.ny >= 32
    assert (out["own"][0] in (1, 2, 4)) == pow2 and out["cufft"][0] == 0
    ev = rel_err(out["own"][1], out["cufft"][1])
    print("%s own vs cuFFT V %.2e" % (name, ev))
    assert ev < 5e-6
    if T is not None:
        assert rel_err(out["own"][2], out["cufft"][2]) < 5e-6


@pytest.mark.parametrize("nx,ny", FUSED)
@pytest.mark.parametrize("planes", [1, 5, 40])
def test_one_launch_equals_two_pass(nx, ny, planes):
    g = torch.Generator(device="cuda").manual_seed(nx + planes)
    x = torch.randn(planes, ny, nx, device="cuda", generator=g, dtype=torch.float32)
    s2 = torch.empty(planes, ny, nx // 2 + 1, dtype=torch.complex64, device="cuda")
    s1 = torch.empty_like(s2)
    _xy(nx, ny, planes, x, s2, False, form=0)
    for _ in range(3):
        s1.fill_(float("nan"))
        _xy(nx, ny, planes, x, s1, False, form=1)
        d = float((s1 - s2).abs().max() / s2.abs().max())
        print("%d x %d x %d forward one-launch vs two-pass %.2e" % (nx, ny, planes, d))
        assert d < 1e-6
    b2 = torch.empty_like(x)
    b1 = torch.empty_like(x)
    _xy(nx, ny, planes, s2.clone(), b2, True, form=0)
    for _ in range(3):
        b1.fill_(float("nan"))
        _xy(nx, ny, planes, s2.clone(), b1, True, form=1)
        d = float((b1 - b2).abs().max() / b2.abs().max())
        print("%d x %d x %d inverse one-launch vs two-pass %.2e" % (nx, ny, planes, d))
        assert d < 1e-6


@pytest.mark.parametrize("nx,ny", CLUSTER)
@pytest.mark.parametrize("planes", [1, 5, 40, 390])
def test_cluster_form_equals_two_pass(nx, ny, planes):
    """The cluster form (a plane across 8 CTAs' shared memory, the column
    pass through distributed shared memory): the two-pass results (same
    arithmetic per value), forward and inverse, on repeated launches, for
    fewer planes than clusters and for several planes per cluster."""
    g = torch.Generator(device="cuda").manual_seed(nx + planes + 1)
    x = torch.randn(planes, ny, nx, device="cuda", generator=g, dtype=torch.float32)
    s2 = torch.empty(planes, ny, nx // 2 + 1, dtype=torch.complex64, device="cuda")
    s1 = torch.empty_like(s2)
    _xy(nx, ny, planes, x, s2, False, form=0)
    for _ in range(2):
        s1.fill_(float("nan"))
        _xy(nx, ny, planes, x, s1, False, form=2)
        d = float((s1 - s2).abs().max() / s2.abs().max())
        print("%d x %d x %d forward cluster vs two-pass %.2e" % (nx, ny, planes, d))
        assert d < 1e-6
    b2 = torch.empty_like(x)
    b1 = torch.empty_like(x)
    _xy(nx, ny, planes, s2.clone(), b2, True, form=0)
    for _ in range(2):
        b1.fill_(float("nan"))
        _xy(nx, ny, planes, s2.clone(), b1, True, form=2)
        d = float((b1 - b2).abs().max() / b2.abs().max())
        print("%d x %d x %d inverse cluster vs two-pass %.2e" % (nx, ny, planes, d))
        assert d < 1e-6


def test_cluster_form_rejects_other_sizes():
    x = torch.zeros(1, 128, 128, device="cuda")
    s = torch.zeros(1, 128, 65, dtype=torch.complex64, device="cuda")
    with pytest.raises(_lib.DPStokesError):
        _xy(128, 128, 1, x, s, False, form=2)


def test_one_launch_rejects_other_sizes():
    x = torch.zeros(1, 64, 128, device="cuda")
    s = torch.zeros(1, 64, 65, dtype=torch.complex64, device="cuda")
    with pytest.raises(_lib.DPStokesError):
        _xy(128, 64, 1, x, s, False, form=1)


@pytest.mark.parametrize("name", ["c2_dp_n65536@128", "c2_dp_n65536@256"])
def test_operator_one_launch_matches_two_pass(name, monkeypatch):
    w = W.by_name(name)
    X, F, T = W.make_inputs(w)
    rng = np.random.default_rng(3)
    K = 3
    Fk = rng.standard_normal((K, w.N, 3)).astype(np.float32)
    Tk = rng.standard_normal((K, w.N, 3)).astype(np.float32)
    out = {}
    for form in ("twopass", "fused", "cluster"):
        if form == "cluster" and w.nx not in (256, 512):
            continue
        monkeypatch.setenv("DPSTOKES_GB300_XY_FFT", form)
        op = DPStokes(StokesParams.from_workload(w, "mixed"), w.N)
        assert op.info()["xy_transform"] == {"fused": 2, "twopass": 1, "cluster": 4}[form]
        op.set_positions(torch.tensor(X, device=op.device))
        V, Wv = op.mdot(torch.tensor(F, dtype=torch.float32, device=op.device),
                        torch.tensor(T, dtype=torch.float32, device=op.device))
        Vk, Wk = op.mdot_multi(torch.tensor(Fk, device=op.device), torch.tensor(Tk, device=op.device))
        torch.cuda.synchronize()
        out[form] = [a.double().cpu().numpy() for a in (V, Wv, Vk, Wk)]
        op.close()
    for a, b in zip(out["fused"], out["twopass"]):
        assert rel_err(a, b) < 5e-6
    if "cluster" in out:
        for a, b in zip(out["cluster"], out["twopass"]):
            assert rel_err(a, b) < 5e-6


@pytest.mark.parametrize("name", ["c0_dpbw_n2048", "c2_dp_n65536@128", "c1_dpsc_n16384@128"])
def test_fp64_operator_double_float_xy_transform(name, monkeypatch):
    """The FP64 operator on the library's double-float x-y transforms against
    the same operator on cuFFT's FP64 transforms (1e-12), and against the
    reference fixture where one exists (1e-10)."""
    import golden_io
    w = W.by_name(name)
    X, F, T = W.make_inputs(w)
    out = {}
    for which in ("own", "cufft"):
        monkeypatch.setenv("DPSTOKES_GB300_XY_FFT", which)
        op = DPStokes(StokesParams.from_workload(w, "fp64"), w.N)
        form = op.info()["xy_transform"]
        op.set_positions(torch.tensor(X, device=op.device))
        V, Wv = op.mdot(torch.tensor(F, device=op.device),
                        torch.tensor(T, device=op.device) if T is not None else None)
        torch.cuda.synchronize()
        out[which] = (form, V.cpu().numpy(), Wv.cpu().numpy() if Wv is not None else None)
        op.close()
    assert out["own"][0] == 3 and out["cufft"][0] == 0
    ev = rel_err(out["own"][1], out["cufft"][1])
    print("%s FP64 own double-float vs cuFFT V %.2e" % (name, ev))
    assert ev < 1e-12
    if T is not None:
        assert rel_err(out["own"][2], out["cufft"][2]) < 1e-12
    if name in golden_io.names():
        _, _, _, _, gd = golden_io.inputs(name)
        assert rel_err(golden_io.restrict(gd, out["own"][1]), gd["V"]) < 1e-10
