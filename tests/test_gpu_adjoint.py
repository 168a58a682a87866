"""The library's discrete adjoint (ib_adjoint_forward / ib_adjoint_backward) for stationary rigid
bodies in a moving frame: its forward against plain steps, its gradient against the oracle's
adjoint (oracle/ib_adjoint.py), against central differences of the GPU forward, for every
checkpoint interval, the context left as the forward left it, and the torch.autograd binding
carrying the gradient to pitching parameters; the same with the Schur system solved by GMRES
(num_stat = F) and its transpose in the reverse, and through the sub-domain method."""
import numpy as np
import pytest

import ib_adjoint as A
import ib_oracle as O
from ib_parallel_gb300 import ibgpu as G

pytestmark = pytest.mark.gpu

KW = dict(m=64, n=32, mgridlev=3, dt=0.01, Re=100.0, len=4.0, offsetx=1.0, offsety=1.0, num_stat=True,
          motion=(-1.0, 0.0, 0.0, 0.3, 0.0), autotune=False)


def _gpu():
    return G.Simulation(G.Params(**KW), [G.Body(**_cyl_kw())])


def _cyl_kw():
    b = O.cylinder(npts=20, diameter=0.8, xc=0.3, yc=0.0)
    return dict(x=b.x.copy(), y=b.y.copy(), fam=1)


def _oracle():
    p = O.Params(**{k: v for k, v in KW.items() if k in O.Params.__dataclass_fields__})
    return O.IBOracle(p, [O.cylinder(npts=20, diameter=0.8, xc=0.3, yc=0.0)])


def _coefs(N):
    t = np.arange(N, dtype=np.float64)
    return np.stack([-1.0 + 0.1 * np.sin(t), 0.2 * np.cos(t), 0.3 * np.sin(0.5 * t)], 1)


def test_forward_is_the_plain_step():
    N = 5
    g = _gpu()
    ref = _gpu()
    forces = g.adjoint_forward(np.tile([-1.0, 0.0, 0.0], (N, 1)), K=2)
    for n in range(N):
        ref.advance()
        cx, cy = ref.forces()
        assert np.allclose(forces[n, 0], [cx[0], cy[0]], rtol=1e-12, atol=0), n
    assert np.allclose(g.get_field("omega", 0), ref.get_field("omega", 0), rtol=0,
                       atol=1e-12 * np.abs(ref.get_field("omega", 0)).max())


def test_gradient_matches_the_oracle_adjoint():
    N = 8
    coefs = _coefs(N)
    W = np.random.default_rng(3).standard_normal((N, 1, 2))
    ad = A.Adjoint(_oracle())
    Fo = ad.forward(coefs)
    go = ad.backward(W)
    g = _gpu()
    Fg = g.adjoint_forward(coefs, K=3)
    gg = g.adjoint_backward(W)
    assert np.abs(Fg - Fo).max() < 1e-10 * np.abs(Fo).max()
    assert np.abs(gg - go).max() < 1e-9 * np.abs(go).max(), np.abs(gg - go).max() / np.abs(go).max()


def test_gradient_matches_central_differences_of_the_gpu_forward():
    N = 8
    coefs = _coefs(N)
    W = np.random.default_rng(4).standard_normal((N, 1, 2))
    g = _gpu()
    g.adjoint_forward(coefs, K=4)
    grad = g.adjoint_backward(W)

    def J(c):
        s = _gpu()
        return float(np.sum(W * s.adjoint_forward(c, K=N)))

    h = 1e-6
    for (n, i) in [(0, 0), (3, 1), (7, 2), (5, 0), (2, 2)]:
        cp = coefs.copy(); cp[n, i] += h
        cm = coefs.copy(); cm[n, i] -= h
        fd = (J(cp) - J(cm)) / (2 * h)
        assert abs(grad[n, i] - fd) <= 1e-6 * max(abs(fd), 1e-3 * np.abs(grad).max()), (n, i, grad[n, i], fd)


@pytest.mark.parametrize("K", [1, 3, 10])
def test_checkpoint_interval_does_not_change_the_gradient(K):
    N = 10
    coefs = _coefs(N)
    W = np.random.default_rng(5).standard_normal((N, 1, 2))
    ref = _gpu()
    ref.adjoint_forward(coefs, K=N)
    g0 = ref.adjoint_backward(W)
    g = _gpu()
    g.adjoint_forward(coefs, K=K)
    assert np.array_equal(g.adjoint_backward(W), g0)


def test_context_continues_from_the_forward():
    N = 4
    coefs = _coefs(N)
    a, b = _gpu(), _gpu()
    a.adjoint_forward(coefs, K=2)
    b.adjoint_forward(coefs, K=2)
    a.adjoint_backward(np.ones((N, 1, 2)))
    a.advance()
    b.advance()
    assert np.array_equal(a.get_field("omega", 0), b.get_field("omega", 0))


def test_autograd_binding_reaches_pitching_parameters():
    torch = pytest.importorskip("torch")
    from ib_parallel_gb300 import autodiff as AD
    N, dt = 12, KW["dt"]

    def mean_lift(amp, freq, phase):
        g = _gpu()
        frames = AD.pitching_frames(N, dt, amp, freq, phase)
        forces = AD.FrameForces.apply(frames, g, 4)
        lift, _ = AD.lift_drag(forces, frames)
        return lift.mean()

    amp = torch.tensor(0.17, dtype=torch.float64, requires_grad=True)
    freq = torch.tensor(0.8, dtype=torch.float64, requires_grad=True)
    phase = torch.tensor(0.3, dtype=torch.float64, requires_grad=True)
    J = mean_lift(amp, freq, phase)
    J.backward()
    h = 1e-6
    for i, p in enumerate((amp, freq, phase)):
        args = [amp.detach().clone(), freq.detach().clone(), phase.detach().clone()]
        args[i] = args[i] + h
        jp = float(mean_lift(*args))
        args[i] = args[i] - 2 * h
        jm = float(mean_lift(*args))
        fd = (jp - jm) / (2 * h)
        assert abs(float(p.grad) - fd) <= 1e-6 * max(abs(fd), 1e-6), (i, float(p.grad), fd)


def test_gradient_at_the_pitching_airfoil_size_matches_the_oracle():
    # the bench's 600x300x4 NACA 0012 in its pitching frame, 4 steps (the oracle's adjoint step at
    # this size takes about a second)
    from ib_parallel_gb300 import autodiff as AD
    from ib_parallel_gb300 import geometry as GEO
    p, bodies = GEO.config_pitching_600x300()
    p.autotune = False
    N = 4
    frames = AD.pitching_frames(N, p.dt, 0.1745, 0.2, 0.0).numpy()
    W = np.random.default_rng(7).standard_normal((N, 1, 2))
    g = G.Simulation(p, bodies)
    Fg = g.adjoint_forward(frames, K=2)
    gg = g.adjoint_backward(W)
    po = O.Params(**{k: getattr(p, k) for k in O.Params.__dataclass_fields__ if hasattr(p, k)})
    o = O.IBOracle(po, [O.Body(x=bodies[0].x.copy(), y=bodies[0].y.copy(), fam=1)])
    ad = A.Adjoint(o)
    Fo = ad.forward(frames)
    go = ad.backward(W)
    assert np.abs(Fg - Fo).max() < 1e-11 * np.abs(Fo).max()
    assert np.abs(gg - go).max() < 1e-10 * np.abs(go).max(), np.abs(gg - go).max() / np.abs(go).max()


# the Schur system by the cluster GMRES on the assembled operator (num_stat = F), both solves tight
KWG = dict(KW, num_stat=False, rtol=1e-14, atol=1e-16)


def _gpu_gmres():
    return G.Simulation(G.Params(**KWG), [G.Body(**_cyl_kw())])


def test_gmres_path_gradient_matches_the_oracle_adjoint():
    # the oracle solves exactly with the dense Schur matrix and reverses with its transpose; the
    # library solves S f = r and S^T x = b by GMRES to 1e-14
    N = 6
    coefs = _coefs(N)
    W = np.random.default_rng(8).standard_normal((N, 1, 2))
    p = O.Params(**{k: v for k, v in KWG.items() if k in O.Params.__dataclass_fields__})
    ad = A.Adjoint(O.IBOracle(p, [O.cylinder(npts=20, diameter=0.8, xc=0.3, yc=0.0)]))
    Fo = ad.forward(coefs)
    go = ad.backward(W)
    g = _gpu_gmres()
    Fg = g.adjoint_forward(coefs, K=2)
    gg = g.adjoint_backward(W)
    assert np.abs(Fg - Fo).max() < 1e-10 * np.abs(Fo).max()
    assert np.abs(gg - go).max() < 1e-8 * np.abs(go).max(), np.abs(gg - go).max() / np.abs(go).max()


def test_gmres_path_gradient_matches_central_differences():
    N = 6
    coefs = _coefs(N)
    W = np.random.default_rng(9).standard_normal((N, 1, 2))
    g = _gpu_gmres()
    g.adjoint_forward(coefs, K=3)
    grad = g.adjoint_backward(W)

    def J(c):
        s = _gpu_gmres()
        return float(np.sum(W * s.adjoint_forward(c, K=N)))

    h = 1e-6
    for (n, i) in [(0, 0), (2, 1), (5, 2), (4, 0)]:
        cp = coefs.copy(); cp[n, i] += h
        cm = coefs.copy(); cm[n, i] -= h
        fd = (J(cp) - J(cm)) / (2 * h)
        assert abs(grad[n, i] - fd) <= 1e-6 * max(abs(fd), 1e-3 * np.abs(grad).max()), (n, i, grad[n, i], fd)


@pytest.mark.parametrize("K", [1, 6])
def test_gmres_path_checkpoint_interval_does_not_change_the_gradient(K):
    # the checkpoints hold the forces too (the next solve's starting guess): a recomputed
    # segment repeats the forward bit for bit
    N = 6
    coefs = _coefs(N)
    W = np.random.default_rng(10).standard_normal((N, 1, 2))
    ref = _gpu_gmres()
    ref.adjoint_forward(coefs, K=2)
    g0 = ref.adjoint_backward(W)
    g = _gpu_gmres()
    g.adjoint_forward(coefs, K=K)
    assert np.array_equal(g.adjoint_backward(W), g0)


# the sub-domain method (sub_domain = T): a small rigid cylinder inside a 13 x 9 cloud
SD_CLOUD = (-0.25, 0.5, -0.25, 0.25, 0.0625)


def _sd_body():
    b = O.cylinder(npts=8, diameter=0.3, xc=0.1, yc=0.0)
    return b, dict(x=b.x.copy(), y=b.y.copy(), fam=1)


def _gpu_sd(path=None):
    g = G.Simulation(G.Params(**KWG), [G.Body(**_sd_body()[1])])
    g.subdomain_setup(*SD_CLOUD)
    if path is not None:
        g.read_subdomain_matrix(path)
    return g


def _sd_matrix(tmp_path):
    g = _gpu_sd()
    g.subdomain_precompute()
    path = tmp_path / "sd_adjoint.chd"
    g.write_subdomain_matrix(path)
    g.close()
    return path


def test_subdomain_gradient_matches_the_oracle_adjoint(tmp_path):
    import ib_subdomain as SD
    path = _sd_matrix(tmp_path)
    N = 5
    coefs = _coefs(N)
    W = np.random.default_rng(11).standard_normal((N, 1, 2))
    p = O.Params(**{k: v for k, v in KWG.items() if k in O.Params.__dataclass_fields__})
    o = O.IBOracle(p, [_sd_body()[0]])
    o.sd = SD.SubDomain(o, True, *SD_CLOUD)
    o.sd.read_chd(path)                  # the same thinned B on both sides
    ad = A.Adjoint(o)
    Fo = ad.forward(coefs)
    go = ad.backward(W)
    g = _gpu_sd(path)
    Fg = g.adjoint_forward(coefs, K=2)
    gg = g.adjoint_backward(W)
    assert np.abs(Fg - Fo).max() < 1e-10 * np.abs(Fo).max()
    assert np.abs(gg - go).max() < 1e-8 * np.abs(go).max(), np.abs(gg - go).max() / np.abs(go).max()


def test_subdomain_gradient_matches_central_differences(tmp_path):
    path = _sd_matrix(tmp_path)
    N = 5
    coefs = _coefs(N)
    W = np.random.default_rng(12).standard_normal((N, 1, 2))
    g = _gpu_sd(path)
    g.adjoint_forward(coefs, K=2)
    grad = g.adjoint_backward(W)

    def J(c):
        s = _gpu_sd(path)
        return float(np.sum(W * s.adjoint_forward(c, K=N)))

    h = 1e-6
    for (n, i) in [(0, 0), (2, 1), (4, 2)]:
        cp = coefs.copy(); cp[n, i] += h
        cm = coefs.copy(); cm[n, i] -= h
        fd = (J(cp) - J(cm)) / (2 * h)
        assert abs(grad[n, i] - fd) <= 1e-6 * max(abs(fd), 1e-3 * np.abs(grad).max()), (n, i, grad[n, i], fd)


def test_subdomain_gradient_at_the_pitching_airfoil_size(tmp_path):
    # the 600x300x4 NACA 0012 in its pitching frame through the sub-domain method (a 56 x 11 cloud
    # at two grid spacings around the chord), GMRES on lumat to 1e-13, 3 steps against the oracle
    import dataclasses
    import ib_subdomain as SD
    from ib_parallel_gb300 import autodiff as AD
    from ib_parallel_gb300 import geometry as GEO
    p, bodies = GEO.config_pitching_600x300()
    p = dataclasses.replace(p, autotune=False, num_stat=False, rtol=1e-13, atol=1e-15)
    cloud = (-0.05, 1.05, -0.1, 0.1, 0.02)
    g = G.Simulation(p, bodies)
    g.subdomain_setup(*cloud)
    g.subdomain_precompute()
    path = tmp_path / "sd_airfoil.chd"
    g.write_subdomain_matrix(path)
    g.close()
    N = 3
    frames = AD.pitching_frames(N, p.dt, 0.1745, 0.2, 0.0).numpy()
    W = np.random.default_rng(13).standard_normal((N, 1, 2))
    g = G.Simulation(p, bodies)
    g.subdomain_setup(*cloud)
    g.read_subdomain_matrix(path)
    Fg = g.adjoint_forward(frames, K=2)
    gg = g.adjoint_backward(W)
    po = O.Params(**{k: getattr(p, k) for k in O.Params.__dataclass_fields__ if hasattr(p, k)})
    o = O.IBOracle(po, [O.Body(x=bodies[0].x.copy(), y=bodies[0].y.copy(), fam=1)])
    o.sd = SD.SubDomain(o, True, *cloud)
    o.sd.read_chd(path)
    ad = A.Adjoint(o)
    Fo = ad.forward(frames)
    go = ad.backward(W)
    assert np.abs(Fg - Fo).max() < 1e-10 * np.abs(Fo).max()
    assert np.abs(gg - go).max() < 1e-8 * np.abs(go).max(), np.abs(gg - go).max() / np.abs(go).max()
