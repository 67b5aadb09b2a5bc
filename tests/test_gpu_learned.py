"""The learned preconditioner end to end on the GPU: pairs harvested from the
method's own multigrid FCG solves along a SIMP trajectory, the U-Net trained
on the GPU with the energy-norm loss, and the learned FCG inside SIMP.

Ablation (what the trained network gains over the method without it):
* one step: the K-norm error of the V-cycle's result after the network's
  correction with its energy-optimal step (as the solver applies it), relative
  to no correction (1), on the training pairs and on held-out pairs from later
  designs, for the trained and an untrained network (printed with -s).
  Asserted: the trained network learned the training distribution (< 0.9) and
  beats the untrained one on the held-out pairs;
* whole solves: the FCG iteration counts of the cycle with the trained network,
  with an untrained one and without a network, all to the FP64 true residual
  1e-8, are recorded (printed with -s); every variant must reach the residual,
  and the trained correction may cost at most twice the iterations of the cycle
  without it (it does not reduce them: the negative result is recorded with its
  experiment matrix in the design notes);
* a stall (a limit below the iterations the learned FCG needs) falls back to the
  FP64 Jacobi PCG, which still reaches the FP64 residual.
"""
import numpy as np
import pytest

from pansfem2_gb300 import problems as PB

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import pansfem2_gb300 as P
    P.load()
    return P


@pytest.fixture(scope="module")
def trained(gpu):
    from pansfem2_gb300 import learned as Ln
    nx, ny = 64, 32
    pr = PB.mbb_q4(nx, ny)
    prob = gpu.Problem(pr)
    prob.setup_bc()
    prob.simp_begin(solver="ir_mg_f32", cg_eps=1e-8, warm_start=True)
    prob.attach_learned(None, pre_mg=True, nu_post=1, use_net=False)
    train = Ln.TrainSet(nx + 1, ny + 1, 320)
    held = Ln.TrainSet(nx + 1, ny + 1, 40)
    for k in range(20):
        prob.simp_step()
        if k % 2 == 1 and k < 16:
            prob.harvest(train, 40, iters=[0, 1, 2, 3, 4, 6, 8, 12, 16, 24])
        if k in (17, 19):
            prob.harvest(held, 20, iters=[0, 1, 2, 4, 8])
    net = Ln.UNet(nx + 1, ny + 1, batch=8, seed=3)
    hist = Ln.train(net, train, 2000, batch=8, lr=1e-3, seed=5, loss="angle")
    yield prob, net, train, held, hist
    prob.close()


def test_training_reduces_the_energy_loss(trained):
    _, _, _, _, hist = trained
    # the scale-free loss starts near 1 (a random direction removes almost no error)
    assert np.isfinite(hist).all()
    assert hist[-100:].mean() < hist[:20].mean() - 0.02
    assert hist[-100:].mean() < 1.0


def test_ablation_one_step_on_held_out_pairs(trained, gpu):
    from pansfem2_gb300 import learned as Ln
    prob, net, train, held, _ = trained
    e_trained = Ln.evaluate(net, held)
    e_train_set = Ln.evaluate(net, train, 0, 40)
    net0 = Ln.UNet(net.H, net.W, batch=8, seed=3)
    net0.out_scale = net.out_scale
    e_untrained = Ln.evaluate(net0, held)
    print(f"relative K-norm error after the correction: trained {e_trained:.3f} (train pairs {e_train_set:.3f}), "
          f"untrained {e_untrained:.3f}, none 1.000")
    assert e_train_set < 0.9
    assert e_trained < e_untrained


def test_ablation_solves_reach_fp64_residual(trained, gpu):
    from pansfem2_gb300 import learned as Ln
    prob, net, _, _, _ = trained
    net0 = Ln.UNet(net.H, net.W, batch=1, seed=3)
    u_mg, i_mg = prob.solve("ir_mg_f32", itmax=20000, eps=1e-8)
    its = {"ir_mg_f32": i_mg["iterations"]}
    for name, n_, kw in (("cycle without network", net, dict(use_net=False)), ("trained network", net, {}),
                         ("untrained network", net0, {})):
        prob.attach_learned(n_, fallback_after=-1, **kw)
        u, info = prob.solve("ir_learned_f32", itmax=5000, eps=1e-8)
        assert info["status"] == 0 and info["rel_residual"] < 1e-8, (name, info)
        assert np.linalg.norm(u - u_mg) <= 1e-5 * np.linalg.norm(u_mg), name
        its[name] = info["iterations"]
    print("FCG iterations to FP64 1e-8:", its)
    # the measured relation (no gain in whole solves; recorded with the experiment matrix in the design
    # notes): the trained correction costs at most twice the iterations of the cycle without it
    assert its["trained network"] <= 2 * its["cycle without network"], its


def test_learned_simp_trajectory_matches_multigrid(trained, gpu):
    """SIMP with the learned solver (fallback enabled) follows the FP64-accurate
    trajectory: compliance within 1e-6, densities within 1e-6 over 10 iterations."""
    prob, net, _, _, _ = trained
    pr = PB.mbb_q4(64, 32)
    runs = {}
    for solver in ("ir_mg_f32", "ir_learned_f32"):
        with gpu.Problem(pr) as P:
            P.setup_bc()
            if solver == "ir_learned_f32":
                P.attach_learned(net, pre_mg=True, nu_post=1)
            P.simp_begin(solver=solver, cg_eps=1e-10)
            f, rho = [], []
            for _ in range(10):
                info = P.simp_step()
                assert info["solve"]["rel_residual"] < 1e-9
                f.append(info["f"])
                rho.append(P.fields()["rho"])
            runs[solver] = (np.array(f), np.array(rho))
    fa, ra = runs["ir_mg_f32"]
    fb, rb = runs["ir_learned_f32"]
    assert np.max(np.abs(fa - fb) / np.abs(fa)) < 1e-6
    assert np.max(np.abs(ra - rb)) < 1e-6


def test_stall_falls_back_to_fp64_jacobi_pcg(trained, gpu):
    """A stall limit below what the learned flexible CG needs (3 iterations) hands the solve to the
    FP64 Jacobi PCG from the current iterate: the solve reports the fallback and still reaches the
    FP64 true residual, with the multigrid solver's answer."""
    prob, net, _, _, _ = trained
    prob.attach_learned(net, pre_mg=True, nu_post=1, fallback_after=3)
    u, info = prob.solve("ir_learned_f32", itmax=100000, eps=1e-8)
    assert info["fell_back"] == 1, info
    assert info["rel_residual"] < 1e-8 and info["iterations"] > 3, info
    u_mg, _ = prob.solve("ir_mg_f32", itmax=20000, eps=1e-10)
    assert np.linalg.norm(u - u_mg) <= 1e-5 * np.linalg.norm(u_mg)
    prob.attach_learned(net, pre_mg=True, nu_post=1)
