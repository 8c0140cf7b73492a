"""The learned KT step: trained on the GPU by the library's own kernels on
(column, sub-cycled KT column) pairs that the plain solver generates, it
gains over the coarse step it corrects; the plain sub-cycled KT kernel is its
fallback and the reference its error is measured against."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_COEF = 3.5 / (2 * 1540.0 ** 3 * 1000.0)
# a Burgers step of 2 mm (CFL numbers up to ~0.45 at these peaks) against the
# same step sub-cycled at CFL 0.01 (up to ~45 sub-cycles)
DZ, DT = 2e-3, 1e-8
CFL = 0.01
MIN_SUB = 10  # learned path from CFL ~0.1 up


def _rel(a, b):
    return float(((a - b) ** 2).sum().sqrt() / ((b ** 2).sum().sqrt() + 1e-30))


@pytest.fixture(scope="module")
def trained():
    from angularspectrum_heterogeneous_gb300 import corrector as CR
    pool = CR.focused_field_columns(6, grid=(64, 64, 512), steps=20, seed=1)
    held = CR.focused_field_columns(1, grid=(64, 64, 512), steps=25, seed=9)
    # peak CFL number 0.35 for the held-out field, so that part of it is learned
    held = (held * (0.35 / (N_COEF / DT * DZ * float(held.abs().max())))).contiguous()
    net = CR.Corrector(CR.init_params(0))
    hist = CR.train(net, pool, N_COEF, DZ, DT, CFL, steps=1500, batch=256, lr=3e-3, seed=0)
    yield CR, net, held, hist
    net.close()


def test_training_converges(trained):
    CR, net, held, hist = trained
    # the scaled targets have unit variance at the start: a quarter is left
    assert np.mean(hist[-20:]) < 0.3 * np.mean(hist[:5]), (hist[:5], hist[-20:])


def test_learned_step_gains_over_the_coarse_step(trained):
    import torch
    CR, net, held, hist = trained
    _, _, _, coarse, fine = CR.training_pairs(held, N_COEF, DZ, DT, CFL)
    out, nl = CR.learned_flux(net, held, N_COEF, DZ, DT, CFL, min_subcycles=MIN_SUB,
                              shock_ratio=1e9)
    cfl = (N_COEF / DT) * held.abs().amax(1) * DZ
    sel = torch.ceil(cfl / CFL) >= MIN_SUB  # the columns the gate sends to the network
    assert abs(nl - int(sel.sum())) <= 2 and nl > 10, (nl, int(sel.sum()))
    e_coarse = _rel(coarse[sel], fine[sel])
    e_learned = _rel(out[sel], fine[sel])
    assert e_learned < 0.5 * e_coarse, (e_coarse, e_learned)
    # end samples are never changed by a KT step
    assert bool((out[:, 0] == held[:, 0]).all()) and bool((out[:, -1] == held[:, -1]).all())


def test_fallback_is_the_plain_sub_cycled_step(trained):
    CR, net, held, hist = trained
    _, _, _, _, fine = CR.training_pairs(held, N_COEF, DZ, DT, CFL)
    for kw in (dict(min_subcycles=10 ** 6, shock_ratio=1e9), dict(min_subcycles=1, shock_ratio=0.0)):
        out, nl = CR.learned_flux(net, held, N_COEF, DZ, DT, CFL, **kw)
        assert nl == 0
        assert bool((out == fine).all())


def test_gate_selects_the_columns_it_should(trained):
    import torch
    CR, net, held, hist = trained
    min_sub, ratio = 20, 0.3
    out, nl = CR.learned_flux(net, held, N_COEF, DZ, DT, CFL, min_subcycles=min_sub,
                              shock_ratio=ratio)
    s = held.abs().amax(1)
    steep = (held[:, 1:] - held[:, :-1]).abs().amax(1)
    cfl = (N_COEF / DT) * s * DZ
    nsub = torch.where(cfl <= CFL, torch.ones_like(cfl), torch.ceil(cfl / CFL))
    want = (nsub >= min_sub) & (steep <= ratio * s)
    assert abs(nl - int(want.sum())) <= max(2, int(want.sum()) // 100), (nl, int(want.sum()))
    _, _, _, _, fine = CR.training_pairs(held, N_COEF, DZ, DT, CFL)
    # columns clearly on the fallback side of the gate (away from its edges)
    plain = (nsub < min_sub - 1) | (steep > 1.01 * ratio * s)
    assert bool((out[plain] == fine[plain]).all())


def test_learned_stage_in_the_march(trained):
    """The learned stage inside the march (asg_set_learned): a 64x64x512
    focused-piston march of 2 mm KT steps whose focal columns need 10-30
    sub-cycles at CFL 0.01.  The plain march sub-cycles every column (its
    FP64 oracle does the same, flux_kt_percolumn); the learned march takes
    one coarse step plus the network's correction on the columns the gate
    selects.  Its pnp/ppp/pI stay within 1e-3 of both; their distances from
    the plain march are printed beside those of the coarse march (one KT
    step per column, no sub-cycling)."""
    import oracle.asm_oracle as O
    import scenarios as S
    from angularspectrum_heterogeneous_gb300 import Plan
    from gpu_helpers import oracle_params, rel, solver_params
    CR, net, held, hist = trained
    nX, nY, nT = 64, 64, 512
    kw = dict(dX=1.5e-4, dY=1.5e-4, dT=DT, c0=1540.0, rho0=1000.0, beta=3.5, alpha0=0.5,
              attenPow=1.0, f0=2e6, dZmin=DZ, propDist=6 * DZ, fluxScheme="kt",
              stabilityThreshold=1.0)
    u0 = S.piston_field(nX, nY, nT, kw["dX"], kw["dY"], kw["dT"], kw["f0"], 1.5e6,
                        radius=0.35 * nX * kw["dX"], focus=10e-3)

    def march(cfl, learned):
        plan = Plan((nX, nY, nT), solver_params(kw), kt_cfl_target=cfl)
        try:
            plan.set_operators(0, DZ)
            if learned:
                plan.set_learned(net, min_subcycles=MIN_SUB, shock_ratio=0.5)
            plan.run(u0, kw["propDist"], DZ)
            return plan.outputs(), plan.learned_stats()
        finally:
            plan.close()

    plain, _ = march(CFL, False)
    learned, (nl, ncs) = march(CFL, True)
    coarse, _ = march(0.0, False)
    assert nl > 0 and ncs == 6 * nX * nY, (nl, ncs)
    ref = O.solve(u0, oracle_params(dict(kw, kt_cfl_target=CFL)), "fp64")
    errs = {}
    for i, k in [(0, "field"), (1, "pnp"), (2, "ppp"), (3, "pI")]:
        errs[k] = dict(plain_vs_fp64=rel(plain[i], ref[i]), learned_vs_plain=rel(learned[i], plain[i]),
                       learned_vs_fp64=rel(learned[i], ref[i]), coarse_vs_plain=rel(coarse[i], plain[i]))
    print(f"\n{nl} learned column steps of {ncs}:",
          {k: {a: f"{b:.2e}" for a, b in v.items()} for k, v in errs.items()})
    for k, e in errs.items():
        bar = 1e-4 if k == "field" else 1e-3
        assert e["plain_vs_fp64"] < bar, (k, e)
        if k != "field":
            assert e["learned_vs_plain"] < 1e-3 and e["learned_vs_fp64"] < 1e-3, (k, e)
