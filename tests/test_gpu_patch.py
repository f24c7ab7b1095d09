"""Parity of the sm_103a patch update against the CPU oracle (GPU required).

Bar (FP64): per step, max |dh|, |dhu|, |dhv| over interior cells within
1e-10 of the depth/momentum scale; wet/dry masks (h > dry_tolerance)
bit-exact; per-patch CFL within 1e-12 relative; total mass within 1e-12
relative. Every case starts both sides from the identical state.
"""
import numpy as np
import pytest

import geoflood_gb300 as gf
import oracle
from geoflood_gb300 import synth

pytestmark = pytest.mark.gpu
MBC = 2
TOL = 1e-10


def scale_of(q):
    return max(1.0, float(np.abs(q).max()))


def compare(q0, out, ref, cfl_gpu, cfl_ref, m, drytol=1e-3, pcfl_gpu=None, pcfl_ref=None):
    s = slice(MBC, MBC + m)
    sc = scale_of(q0[:, s, s])
    err = np.abs(out[:, s, s] - ref[:, s, s]).max(axis=(0, 1, 2))
    assert np.all(err <= TOL * sc), f"max |d(h,hu,hv)| = {err}, scale {sc}"
    assert np.array_equal(out[:, s, s, 0] > drytol, ref[:, s, s, 0] > drytol), "wet/dry mask"
    assert abs(cfl_gpu - cfl_ref) <= 1e-12 * max(1.0, cfl_ref), (cfl_gpu, cfl_ref)
    m_gpu, m_ref = out[:, s, s, 0].sum(), ref[:, s, s, 0].sum()
    assert abs(m_gpu - m_ref) <= 1e-12 * max(1.0, abs(m_ref))
    if pcfl_gpu is not None:
        assert np.allclose(pcfl_gpu, pcfl_ref, rtol=1e-12, atol=1e-300)
    return err


def level_vs_oracle(ctx, q, aux, m, dx, dt, phys, slot=0):
    n = q.shape[0]
    ctx.set_phys(slot, phys)
    lev = gf.Level(ctx, n, m, aux.shape[-1])
    lev.set_geometry(dx, dx, slot)
    lev.upload(q, aux)
    cfl_gpu = lev.step(0.0, dt)
    out = lev.download()
    pc_gpu = lev.patch_cfl()
    lev.close()
    ref = q.copy()
    pc_ref = np.array([oracle.patch_update(ref[k], aux[k], dx, dx, 0.0, dt, phys)
                       for k in range(n)])
    cfl_ref = pc_ref.max() if n else 0.0
    return out, ref, cfl_gpu, cfl_ref, pc_gpu, pc_ref


def random_state(n, m, seed, relief=8.0, depth=3.0, vel=2.0, dx=2.0):
    """Independent patches: fractal terrain, a rough water surface that leaves
    dry islands, random velocities u, v ~ N(0, vel) m/s (hu = h u), ghost cells
    included."""
    g = synth.rng(seed)
    q = np.zeros((n, m + 4, m + 4, 3))
    aux = np.zeros((n, m + 4, m + 4, 1))
    for k in range(n):
        b = synth.fractal_dem(m + 4, m + 4, dx, 0.75, relief, seed * 1000 + k)
        eta = depth + 0.5 * g.standard_normal()
        h = np.maximum(eta - b + 0.3 * g.standard_normal(b.shape), 0.0)
        h[g.random(b.shape) < 0.05] = 0.0
        q[k, ..., 0] = h
        q[k, ..., 1] = h * vel * g.standard_normal(b.shape)
        q[k, ..., 2] = h * vel * g.standard_normal(b.shape)
        aux[k, ..., 0] = b
    return q, aux


@pytest.mark.parametrize("m", [8, 16, 32])
@pytest.mark.parametrize("seed", [1, 2])
def test_dam_break_level(ctx, m, seed):
    q, aux, _, _ = synth.uniform_dam_break_level(4, 4, m, 1.0, seed=seed, x_dam=1.5 * m)
    out, ref, cg, cr, pg, pr = level_vs_oracle(ctx, q, aux, m, 1.0, 0.05, gf.Phys())
    compare(q, out, ref, cg, cr, m, pcfl_gpu=pg, pcfl_ref=pr)


@pytest.mark.parametrize("m", [8, 16, 32])
@pytest.mark.parametrize("seed", [3, 4, 5])
def test_random_wet_dry_patches(ctx, m, seed):
    q, aux = random_state(24, m, seed)
    out, ref, cg, cr, pg, pr = level_vs_oracle(ctx, q, aux, m, 2.0, 0.04, gf.Phys())
    compare(q, out, ref, cg, cr, m, pcfl_gpu=pg, pcfl_ref=pr)


@pytest.mark.parametrize("variant", [
    dict(order=1), dict(transverse=0), dict(transverse=1), dict(order=1, transverse=1),
    dict(mthlim=(1, 1, 1)), dict(mthlim=(2, 2, 2)), dict(mthlim=(3, 3, 3)),
    dict(mthlim=(0, 4, 1)), dict(friction_forcing=False),
    dict(src_term=0), dict(manning_coefficient=(0.06, 0.03), manning_break=(2.0, 1e10)),
    dict(dry_tolerance=1e-2), dict(friction_depth=1.5),
])
def test_method_variants(ctx, variant):
    """Bounded limiters and method switches at the 1e-10 bar. (The unbounded
    Beam-Warming limiter, philim = r, amplifies a 1-ulp input change to
    ~1e-2 in the oracle itself, so it is checked bitwise in the exact build
    instead: test_exact_build_beam_warming.)"""
    m = 16
    q, aux = random_state(12, m, 9)
    out, ref, cg, cr, pg, pr = level_vs_oracle(ctx, q, aux, m, 2.0, 0.04, gf.Phys(**variant),
                                               slot=3)
    compare(q, out, ref, cg, cr, m, drytol=gf.Phys(**variant).dry_tolerance,
            pcfl_gpu=pg, pcfl_ref=pr)


def test_variable_friction_field(ctx):
    m = 16
    q, aux1 = random_state(10, m, 13)
    g = synth.rng(5)
    nfield = np.where(g.random(aux1.shape[:3]) < 0.5, 0.03, 0.07)
    aux = np.concatenate([aux1, nfield[..., None]], axis=-1)
    phys = gf.Phys(variable_friction=True, friction_index=2)
    out, ref, cg, cr, pg, pr = level_vs_oracle(ctx, q, aux, m, 2.0, 0.04, phys, slot=4)
    compare(q, out, ref, cg, cr, m, pcfl_gpu=pg, pcfl_ref=pr)


def test_lake_at_rest_level(ctx):
    m = 32
    b = synth.fractal_dem(4 * m, 4 * m, 5.0, 0.8, 30.0, 21)
    h = np.maximum(12.0 - b, 0.0)
    qg = np.zeros(b.shape + (3,))
    qg[..., 0] = h
    q = synth.tile_level(synth.pad_extrap(qg), m)
    aux = synth.tile_level(synth.pad_extrap(b[..., None]), m)
    out, ref, cg, cr, pg, pr = level_vs_oracle(ctx, q, aux, m, 5.0, 0.3, gf.Phys())
    compare(q, out, ref, cg, cr, m, pcfl_gpu=pg, pcfl_ref=pr)
    s = slice(MBC, MBC + m)
    assert np.abs(out[:, s, s, 1:]).max() < 1e-12


def test_all_dry_level_is_unchanged(ctx):
    m = 16
    q, aux = random_state(6, m, 17)
    q[..., 0] = np.minimum(q[..., 0], 5e-4)
    out, ref, cg, cr, pg, pr = level_vs_oracle(ctx, q, aux, m, 2.0, 0.04, gf.Phys())
    compare(q, out, ref, cg, cr, m)
    assert cg == 0.0 and cr == 0.0


def test_cfl_cap_reports_zero(ctx):
    m = 8
    q, aux = random_state(4, m, 23, vel=40.0)
    q[..., 0] = np.maximum(q[..., 0], 0.5)
    out, ref, cg, cr, pg, pr = level_vs_oracle(ctx, q, aux, m, 0.01, 2.0,
                                               gf.Phys(maxcfl_cap=100.0))
    assert cr == 0.0 and cg == 0.0
    assert np.array_equal(pg, pr)


def test_plain_per_patch_dropin(ctx):
    """gf_patch_update with a host Fortran-layout patch: interior matches the
    oracle, ghost cells come back as they went in."""
    m = 32
    q, aux = random_state(3, m, 31)
    ctx.set_phys(0, gf.Phys())
    for k in range(3):
        qk = q[k].copy()
        cfl = ctx.patch_update(qk, aux[k].copy(), 2.0, 2.0, 0.0, 0.04)
        ref = q[k].copy()
        cfl_ref = oracle.patch_update(ref, aux[k], 2.0, 2.0, 0.0, 0.04)
        compare(q[k:k + 1], qk[None], ref[None], cfl, cfl_ref, m)
        ring = np.ones((m + 4, m + 4), bool)
        ring[MBC:MBC + m, MBC:MBC + m] = False
        assert np.array_equal(qk[ring], q[k][ring])


def test_batched_dropin(ctx):
    m = 16
    q, aux = random_state(20, m, 37)
    ctx.set_phys(0, gf.Phys())
    qs = [q[k].copy() for k in range(20)]
    pc, mc = ctx.patch_update_batch(qs, [aux[k] for k in range(20)], 2.0, 2.0, 0.0, 0.04)
    ref = q.copy()
    pr = np.array([oracle.patch_update(ref[k], aux[k], 2.0, 2.0, 0.0, 0.04) for k in range(20)])
    compare(q, np.stack(qs), ref, mc, pr.max(), m, pcfl_gpu=pc, pcfl_ref=pr)


def test_step_host_equals_resident_step(ctx):
    m = 16
    q, aux = random_state(8, m, 41)
    ctx.set_phys(0, gf.Phys())
    lev = gf.Level(ctx, 8, m)
    lev.set_geometry(2.0, 2.0)
    lev.upload(q, aux)
    c1 = lev.step(0.0, 0.04)
    a = lev.download()
    lev.upload(q)
    qh = q.copy()
    c2 = lev.step_host(qh, 0.0, 0.04)
    s = slice(MBC, MBC + m)
    assert c1 == c2
    assert np.array_equal(a[:, s, s], qh[:, s, s])


def test_deterministic_repeat(ctx):
    m = 32
    q, aux = random_state(8, m, 43)
    ctx.set_phys(0, gf.Phys())
    lev = gf.Level(ctx, 8, m)
    lev.set_geometry(2.0, 2.0)
    outs = []
    for _ in range(3):
        lev.upload(q, aux)
        lev.step(0.0, 0.04)
        outs.append(lev.download())
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[1], outs[2])


def test_multistep_dam_break_resynced(ctx):
    """Ten steps of the uniform-level dam break with ghost cells refilled from
    the global state between steps; each step compared from the GPU state."""
    m, npx, dx, dt = 16, 4, 1.0, 0.05
    q, aux, py, px = synth.uniform_dam_break_level(npx, npx, m, dx, seed=3, x_dam=24.0)
    ctx.set_phys(0, gf.Phys())
    lev = gf.Level(ctx, q.shape[0], m)
    lev.set_geometry(dx, dx)
    lev.upload(q, aux)
    for step in range(10):
        ref = q.copy()
        cr = oracle.level_update(ref, aux, dx, dx, 0.0, dt, gf.Phys(), nthreads=1)
        cg = lev.step(0.0, dt)
        out = lev.download()
        compare(q, out, ref, cg, cr, m)
        glob = synth.untile_level(out, py, px)
        q = synth.tile_level(synth.pad_extrap(glob), m)
        lev.upload(q)


@pytest.fixture
def exact_ctx(gpu_lib):
    c = gf.Context(0)
    c.set_fp_contract(False)
    yield c
    c.close()


@pytest.mark.parametrize("m", [8, 16, 32])
@pytest.mark.parametrize("seed", [51, 52])
def test_exact_build_is_bitwise_without_friction(exact_ctx, m, seed):
    """Contraction off + reference summation order: every interior value equals
    the oracle's bit for bit (no pow() in play)."""
    q, aux = random_state(16, m, seed)
    phys = gf.Phys(friction_forcing=False)
    out, ref, cg, cr, pg, pr = level_vs_oracle(exact_ctx, q, aux, m, 2.0, 0.04, phys, slot=5)
    s = slice(MBC, MBC + m)
    assert np.array_equal(out[:, s, s], ref[:, s, s])
    assert cg == cr and np.array_equal(pg, pr)


@pytest.mark.parametrize("m", [16, 32])
def test_exact_build_depth_bitwise_with_friction(exact_ctx, m):
    """With Manning friction only the momenta see CUDA's pow() against libm's."""
    q, aux, _, _ = synth.uniform_dam_break_level(4, 4, m, 1.0, seed=61, x_dam=1.5 * m)
    out, ref, cg, cr, pg, pr = level_vs_oracle(exact_ctx, q, aux, m, 1.0, 0.05, gf.Phys(), slot=6)
    s = slice(MBC, MBC + m)
    assert np.array_equal(out[:, s, s, 0], ref[:, s, s, 0])
    rel = np.abs(out[:, s, s, 1:] - ref[:, s, s, 1:]) / np.maximum(np.abs(ref[:, s, s, 1:]), 1e-300)
    assert rel.max() < 1e-14


def test_exact_build_beam_warming(exact_ctx):
    m = 16
    q, aux = random_state(12, m, 9)
    phys = gf.Phys(mthlim=(5, 5, 5), friction_forcing=False)
    out, ref, cg, cr, pg, pr = level_vs_oracle(exact_ctx, q, aux, m, 2.0, 0.04, phys, slot=7)
    s = slice(MBC, MBC + m)
    assert np.array_equal(out[:, s, s], ref[:, s, s])


@pytest.mark.parametrize("shuffle", [False, True])
def test_step_host_pipeline_chunks_give_identical_results(ctx, shuffle):
    """gf_level_step_host in 1, 3 or 7 chunks, and the automatic choice, on a
    12 x 10 brick with a layout (ghost fill in the pipeline), patches either
    row-major or shuffled so that a chunk's ghost cells read far chunks: q
    (ghost cells included) and the CFL equal the resident step's bit for bit.
    A first ghost fill makes the aux ghost cells consistent (a fill rewrites
    them), so every step below sees the same bathymetry."""
    m, py, px = 16, 10, 12
    n = py * px
    q, aux = random_state(n, m, 59)
    nbr, xl, yl = synth.brick_layout(py, px, m, 2.0)
    if shuffle:
        perm = np.random.default_rng(5).permutation(n)     # new index -> old index
        inv = np.empty(n, np.int64)
        inv[perm] = np.arange(n)
        q, aux, xl, yl = q[perm], aux[perm], xl[perm], yl[perm]
        nb = nbr[perm]
        nbr = np.where(nb >= 0, inv[np.maximum(nb, 0)], -1).astype(np.int32)
    ctx.set_phys(0, gf.Phys())
    lev = gf.Level(ctx, n, m)
    lev.set_geometry(2.0, 2.0)
    lev.set_layout(nbr, xl, yl)
    lev.upload(q, aux)
    lev.ghost_fill(0.0)
    q0 = lev.download()
    c_ref = lev.step(0.0, 0.04)
    lev.ghost_fill(0.04)
    ref = lev.download()
    for chunks in (1, 3, 7, 0):
        lev.set_pipeline(chunks)
        qh = q0.copy()
        c = lev.step_host(qh, 0.0, 0.04)
        assert c == c_ref, chunks
        assert np.array_equal(qh, ref), chunks
    lev.close()
