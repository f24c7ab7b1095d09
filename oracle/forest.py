"""CPU oracle for multi-level forests -- TEST INFRASTRUCTURE ONLY.

A plain-Python restatement of the forest rules (leaves, 2:1 balance, ghost
exchange between levels, regrid, initial refinement, outstyle-1 stepping)
on top of the oracle's C kernels, which restate the reference's Fortran:
copies and bc2 (fclaw2d_source/fc2d_geoclaw_copy_fort.f,
fortran_source/geoflood_bc2_fort.f90), averaging and interpolation
(fclaw2d_source/fc2d_geoclaw_average_fort.f,
fclaw2d_source/fc2d_geoclaw_interpolate_fort.f), tags
(fclaw2d_source/fc2d_geoclaw_tag4refinement_fort.f90,
fc2d_geoclaw_tag4coarsening_fort.f90) and the patch update. The level
machinery itself belongs to ForestClaw / p4est, which the reference tree
does not contain, so this driver states the rules the device driver
follows; its agreement with ForestClaw is unpinned.
"""
from __future__ import annotations

import os

import numpy as np

from . import (MBC, average2coarse, average_ghost, interpolate2fine, interpolate_ghost,
               level_ghost_fill, level_update, params, refine as c_refine, tag4coarsening,
               tag4refinement)
from . import output as fout

FACES = ((-1, 0), (1, 0), (0, -1), (0, 1))          # left, right, bottom, top
CORNERS = ((-1, -1), (1, -1), (-1, 1), (1, 1))       # ll, lr, ul, ur


def pyramid(fields: np.ndarray, levels: int) -> list:
    """fields (nf, ny, nx) at the finest level -> [finest, ..., coarsest],
    each (nf, ny_l + 4, nx_l + 4) padded by edge copies; coarser interiors are
    ((a + b) + (c + d)) * 0.25 of the 2 x 2 block below."""
    out = []
    cur = np.asarray(fields, np.float64)
    for k in range(levels):
        out.append(np.pad(cur, ((0, 0), (MBC, MBC), (MBC, MBC)), mode="edge"))
        if k + 1 < levels:
            cur = ((cur[:, 0::2, 0::2] + cur[:, 0::2, 1::2])
                   + (cur[:, 1::2, 0::2] + cur[:, 1::2, 1::2])) * 0.25
    return out


class Forest:
    def __init__(self, mx, nbx, nby, minlevel, maxlevel, dx0, dy0, aux, q, x0=0.0, y0=0.0,
                 phys=None, mthbc=(1, 1, 1, 1), regrid_interval=0, rf=None, hy=None,
                 subcycle=False):
        self.subcycle = bool(subcycle)
        self.m, self.nbx, self.nby = mx, nbx, nby
        self.lmin, self.lmax = minlevel, maxlevel
        self.dx0, self.dy0, self.x0, self.y0 = dx0, dy0, x0, y0
        self.phys, self.mthbc, self.hy = phys, tuple(mthbc), hy
        self.regrid_interval = regrid_interval
        self.rf = c_refine(rf) if rf is not None else None
        aux = np.asarray(aux, np.float64)
        if aux.ndim == 2:
            aux = aux[None]
        self.maux = aux.shape[0]
        fields = np.concatenate([aux, np.moveaxis(np.asarray(q, np.float64), 2, 0)], axis=0)
        pyr = pyramid(fields, maxlevel - minlevel + 1)
        self.pyr = {maxlevel - k: p for k, p in enumerate(pyr)}
        self.leaves = {}            # (l, I, J) -> [q (n4, n4, 3), aux (n4, n4, maux)]
        self.steps = self.rejects = self.regrids = 0
        self.cell_updates = 0
        self.t = 0.0
        self.dt = 0.0
        self.max_cfl_seen = 0.0
        self.out_dir, self.frames, self.next_frame, self.out_started = "", False, 0, False
        self.gauges = []            # dicts: id, x, y, t1, t2, incr, last, rows

    def set_topo(self, topo_set, qinit=True):
        """Bathymetry of every level from topo grids (setaux per level, see
        oracle/topo.py) and, with qinit, h = max(0, sea_level - b), hu = hv = 0
        (fortran_source/geoclaw_qinit_fort.f90:24-27)."""
        xu = self.x0 + (self.nbx * self.m) * self.dx0
        yu = self.y0 + (self.nby * self.m) * self.dy0
        sea = params(self.phys).sea_level
        for l in range(self.lmin, self.lmax + 1):
            nx, ny = self.npx(l) * self.m, self.npy(l) * self.m
            b = topo_set.raster(nx, ny, MBC, self.x0, self.y0, self.dx(l), self.dy(l), xu, yu)
            p = self.pyr[l]
            p[0] = b
            if qinit:
                p[self.maux] = np.maximum(0.0, sea - b)
                p[self.maux + 1] = 0.0
                p[self.maux + 2] = 0.0

    # ---- geometry -------------------------------------------------------
    def npx(self, l):
        return self.nbx << l

    def npy(self, l):
        return self.nby << l

    def inside(self, l, I, J):
        return 0 <= I < self.npx(l) and 0 <= J < self.npy(l)

    def dx(self, l):
        return self.dx0 / (1 << l)

    def dy(self, l):
        return self.dy0 / (1 << l)

    def origin(self, l, I, J):
        return (self.x0 + I * self.m * self.dx(l), self.y0 + J * self.m * self.dy(l))

    def containing(self, l, I, J):
        for k in range(l, self.lmin - 1, -1):
            key = (k, I >> (l - k), J >> (l - k))
            if key in self.leaves:
                return key
        return None

    def canonical(self):
        return sorted(self.leaves, key=lambda k: (k[0], k[2], k[1]))

    def window(self, l, I, J):
        n4 = self.m + 2 * MBC
        p = self.pyr[l]
        w = p[:, J * self.m:J * self.m + n4, I * self.m:I * self.m + n4]
        return np.ascontiguousarray(np.moveaxis(w, 0, 2))   # (n4, n4, nf)

    def new_patch(self, key, with_q):
        w = self.window(*key)
        aux = np.ascontiguousarray(w[..., :self.maux])
        q = np.ascontiguousarray(w[..., self.maux:]) if with_q else np.zeros(w.shape[:2] + (3,))
        return [q, aux]

    # ---- ghost exchange -------------------------------------------------
    def _level_fill(self, l, t, arrays=None):
        """Same-level copies and physical sides of level l; arrays (key -> q)
        replaces the leaves' own states when given."""
        keys = [k for k in self.canonical() if k[0] == l]
        if not keys:
            return
        pos = {k: n for n, k in enumerate(keys)}
        nbr = -np.ones((len(keys), 8), np.int32)
        for n, (_, I, J) in enumerate(keys):
            for s, (di, dj) in enumerate(FACES + CORNERS):
                if not self.inside(l, I + di, J + dj):
                    nbr[n, s] = -1
                else:
                    nbr[n, s] = pos.get((l, I + di, J + dj), -2)
        qof = (lambda k: arrays[k]) if arrays is not None else (lambda k: self.leaves[k][0])
        q = np.stack([qof(k) for k in keys])
        aux = np.stack([self.leaves[k][1] for k in keys])
        xl = np.array([self.origin(*k)[0] for k in keys])
        yl = np.array([self.origin(*k)[1] for k in keys])
        level_ghost_fill(q, aux, nbr, xl, yl, self.dx(l), self.dy(l), t, self.mthbc, self.phys,
                         self.hy)
        for n, k in enumerate(keys):
            qof(k)[...] = q[n]
            self.leaves[k][1][...] = aux[n]

    def ghost_fill(self, t):
        m = self.m
        # (1) fine -> coarse averages into coarse ghost cells
        for (l, I, J), (qc, ac) in self.leaves.items():
            for fc, (di, dj) in enumerate(FACES):
                NI, NJ = I + di, J + dj
                if not self.inside(l, NI, NJ) or (l, NI, NJ) in self.leaves:
                    continue
                if l > self.lmin and (l - 1, NI >> 1, NJ >> 1) in self.leaves:
                    continue
                for c in range(2):
                    if fc < 2:
                        FI, FJ = 2 * NI + (1 if di < 0 else 0), 2 * J + c
                    else:
                        FI, FJ = 2 * I + c, 2 * NJ + (1 if dj < 0 else 0)
                    qf, af = self.leaves[(l + 1, FI, FJ)]
                    average_ghost(qc, ac, qf, af, 0, fc, m * (2 * I - FI), m * (2 * J - FJ),
                                  self.phys)
            for cc, (di, dj) in enumerate(CORNERS):
                DI, DJ = I + di, J + dj
                if not self.inside(l, DI, DJ) or (l, DI, DJ) in self.leaves:
                    continue
                if self.containing(l, DI, DJ) is not None:
                    continue
                FI, FJ = 2 * DI + (1 if di < 0 else 0), 2 * DJ + (1 if dj < 0 else 0)
                qf, af = self.leaves[(l + 1, FI, FJ)]
                average_ghost(qc, ac, qf, af, 1, cc, m * (2 * I - FI), m * (2 * J - FJ), self.phys)
        # (2) same-level copies and physical boundaries, every level
        for l in range(self.lmin, self.lmax + 1):
            self._level_fill(l, t)
        # (3) coarse -> fine interpolation, level by level, boundaries again
        for l in range(self.lmin + 1, self.lmax + 1):
            for (lp, I, J), (qf, af) in self.leaves.items():
                if lp != l:
                    continue
                for fc, (di, dj) in enumerate(FACES):
                    NI, NJ = I + di, J + dj
                    if not self.inside(l, NI, NJ) or (l, NI, NJ) in self.leaves:
                        continue
                    ck = (l - 1, NI >> 1, NJ >> 1)
                    if ck in self.leaves:
                        qc, ac = self.leaves[ck]
                        interpolate_ghost(qc, ac, qf, af, 0, fc ^ 1, m * (2 * ck[1] - I),
                                          m * (2 * ck[2] - J), self.phys)
                for cc, (di, dj) in enumerate(CORNERS):
                    DI, DJ = I + di, J + dj
                    if not self.inside(l, DI, DJ) or (l, DI, DJ) in self.leaves:
                        continue
                    ck = (l - 1, DI >> 1, DJ >> 1)
                    if ck not in self.leaves:
                        continue
                    xok = 2 * ck[1] == DI if di > 0 else 2 * ck[1] + 1 == DI
                    yok = 2 * ck[2] == DJ if dj > 0 else 2 * ck[2] + 1 == DJ
                    if xok and yok:
                        qc, ac = self.leaves[ck]
                        interpolate_ghost(qc, ac, qf, af, 1, 3 - cc, m * (2 * ck[1] - I),
                                          m * (2 * ck[2] - J), self.phys)
            self._level_fill(l, t)

    # ---- subcycling ---------------------------------------------------------
    # The level-by-level schedule the device forest follows with subcycle = 1
    # (ForestClaw's fclaw2d_advance_all_levels, an external library: this is
    # the project's statement of it): coarse before fine; a level's two
    # sub-steps inside its parent's step take their coarse ghost values from
    # the parent's start state and from the parent time-interpolated to the
    # midpoint (fc2d_geoclaw_fort_timeinterp on the two layers along each
    # face, the old ghost ring kept, ghost cells exchanged at the midpoint).
    def _avg_level(self, l, qc_of):
        """fine (level l + 1) -> coarse averages into level-l ghost cells;
        qc_of(key) gives the coarse array to write."""
        m = self.m
        for (lv, I, J) in self.canonical():
            if lv != l:
                continue
            qc, ac = qc_of((lv, I, J)), self.leaves[(lv, I, J)][1]
            for fc, (di, dj) in enumerate(FACES):
                NI, NJ = I + di, J + dj
                if not self.inside(l, NI, NJ) or (l, NI, NJ) in self.leaves:
                    continue
                if l > self.lmin and (l - 1, NI >> 1, NJ >> 1) in self.leaves:
                    continue
                for c in range(2):
                    if fc < 2:
                        FI, FJ = 2 * NI + (1 if di < 0 else 0), 2 * J + c
                    else:
                        FI, FJ = 2 * I + c, 2 * NJ + (1 if dj < 0 else 0)
                    qf, af = self.leaves[(l + 1, FI, FJ)]
                    average_ghost(qc, ac, qf, af, 0, fc, m * (2 * I - FI), m * (2 * J - FJ),
                                  self.phys)
            for cc, (di, dj) in enumerate(CORNERS):
                DI, DJ = I + di, J + dj
                if not self.inside(l, DI, DJ) or (l, DI, DJ) in self.leaves:
                    continue
                if self.containing(l, DI, DJ) is not None:
                    continue
                FI, FJ = 2 * DI + (1 if di < 0 else 0), 2 * DJ + (1 if dj < 0 else 0)
                qf, af = self.leaves[(l + 1, FI, FJ)]
                average_ghost(qc, ac, qf, af, 1, cc, m * (2 * I - FI), m * (2 * J - FJ), self.phys)

    def _interp_level(self, l, qc_of):
        """coarse (level l - 1, arrays from qc_of) -> fine ghost cells of level l."""
        m = self.m
        for (lp, I, J), (qf, af) in self.leaves.items():
            if lp != l:
                continue
            for fc, (di, dj) in enumerate(FACES):
                NI, NJ = I + di, J + dj
                if not self.inside(l, NI, NJ) or (l, NI, NJ) in self.leaves:
                    continue
                ck = (l - 1, NI >> 1, NJ >> 1)
                if ck in self.leaves:
                    interpolate_ghost(qc_of(ck), self.leaves[ck][1], qf, af, 0, fc ^ 1,
                                      m * (2 * ck[1] - I), m * (2 * ck[2] - J), self.phys)
            for cc, (di, dj) in enumerate(CORNERS):
                DI, DJ = I + di, J + dj
                if not self.inside(l, DI, DJ) or (l, DI, DJ) in self.leaves:
                    continue
                ck = (l - 1, DI >> 1, DJ >> 1)
                if ck not in self.leaves:
                    continue
                xok = 2 * ck[1] == DI if di > 0 else 2 * ck[1] + 1 == DI
                yok = 2 * ck[2] == DJ if dj > 0 else 2 * ck[2] + 1 == DJ
                if xok and yok:
                    interpolate_ghost(qc_of(ck), self.leaves[ck][1], qf, af, 1, 3 - cc,
                                      m * (2 * ck[1] - I), m * (2 * ck[2] - J), self.phys)

    def _fill_level_sub(self, l, t, csrc, hi):
        own = lambda k: self.leaves[k][0]  # noqa: E731
        if l < hi:
            self._avg_level(l, own)
        self._level_fill(l, t)
        if csrc is not None:
            self._interp_level(l, csrc.__getitem__)
            self._level_fill(l, t)

    def _update_level(self, l, dt):
        keys = [k for k in self.canonical() if k[0] == l]
        q = np.stack([self.leaves[k][0] for k in keys])
        aux = np.stack([self.leaves[k][1] for k in keys])
        dx = np.array([self.dx(l)] * len(keys))
        dy = np.array([self.dy(l)] * len(keys))
        cfl = level_update(q, aux, dx, dy, 0.0, dt, self.phys)
        for n, k in enumerate(keys):
            self.leaves[k][0][...] = q[n]
        return cfl

    def _sub_level(self, l, tl, dtl, hi):
        keys = [k for k in self.canonical() if k[0] == l]
        old = {k: self.leaves[k][0].copy() for k in keys}
        cfl = self._update_level(l, dtl)
        if l >= hi:
            return cfl
        m = self.m
        i = np.arange(m + 4) - 1                      # Fortran index of each array column
        d = np.minimum(np.minimum(i[None, :] - 1, i[:, None] - 1), np.minimum(m - i[None, :], m - i[:, None]))
        strip = (d < 2) & (i[None, :] >= 1) & (i[None, :] <= m) & (i[:, None] >= 1) & (i[:, None] <= m)
        for k in (0, 1):
            tf = tl + dtl * 0.5 if k else tl
            src = old
            if k == 1:
                qi = {}
                for key in keys:
                    a, b = old[key], self.leaves[key][0]
                    qi[key] = a.copy()
                    qi[key][strip] = a[strip] + 0.5 * (b[strip] - a[strip])
                self._avg_level(l, qi.__getitem__)
                self._level_fill(l, tf, arrays=qi)
                src = qi
            self._fill_level_sub(l + 1, tf, src, hi)
            cfl = max(cfl, self._sub_level(l + 1, tf, dtl * 0.5, hi))
        return cfl

    def step_subcycled(self, t, dt):
        """One coarse step dt with subcycling; returns the max CFL of all
        sub-steps and the number of cell-updates."""
        levels = sorted({k[0] for k in self.leaves})
        lo, hi = levels[0], levels[-1]
        self._fill_level_sub(lo, t, None, hi)
        cfl = self._sub_level(lo, t, dt, hi)
        cu = sum(self.m * self.m << (k[0] - lo) for k in self.leaves)
        return cfl, cu

    # ---- tags, balance, regrid ------------------------------------------
    def _tags(self, t, init_flag):
        refine = {}
        for k in self.canonical():
            l, I, J = k
            if l >= self.lmax:
                continue
            q, aux = self.leaves[k]
            xl, yl = self.origin(*k)
            refine[k] = tag4refinement(q, aux, xl, yl, self.dx(l), self.dy(l), t, l, self.lmax,
                                       init_flag, self.rf, self.phys) != 0
        fams = []
        if not init_flag:
            for k in self.canonical():
                l, I, J = k
                if l <= self.lmin or I & 1 or J & 1:
                    continue
                fam = [(l, I + (c & 1), J + (c >> 1)) for c in range(4)]
                if not all(f in self.leaves for f in fam):
                    continue
                qs = [self.leaves[f][0] for f in fam]
                auxs = [self.leaves[f][1] for f in fam]
                xs = [self.origin(*f)[0] for f in fam]
                ys = [self.origin(*f)[1] for f in fam]
                c = tag4coarsening(qs, auxs, xs, ys, self.dx(l), self.dy(l), t, l, self.lmax,
                                   init_flag, self.rf, self.phys)
                fams.append((fam, c != 0))
        return refine, fams

    def _balance(self, split):
        """Split every leaf that a split neighbour's children would touch
        across a two-level jump (face or corner), until none is left."""
        work = [k for k in split]
        while work:
            l, I, J = work.pop()
            for di, dj in FACES + CORNERS:
                if not self.inside(l, I + di, J + dj):
                    continue
                q = self.containing(l, I + di, J + dj)
                if q is not None and q[0] <= l - 1 and q not in split:
                    split.add(q)
                    work.append(q)

    def _can_merge(self, l, PI, PJ, split):
        for a in range(-1, 3):
            for b in range(-1, 3):
                if 0 <= a <= 1 and 0 <= b <= 1:
                    continue
                I, J = 2 * PI + a, 2 * PJ + b
                if not self.inside(l, I, J):
                    continue
                q = self.containing(l, I, J)
                if q is None or (q[0] == l and q in split):
                    return False
        return True

    def _apply(self, split, merges, init):
        new = {}
        for k, (q, aux) in self.leaves.items():
            if k in split:
                l, I, J = k
                for c in range(4):
                    ck = (l + 1, 2 * I + (c & 1), 2 * J + (c >> 1))
                    child = self.new_patch(ck, init)
                    if not init:
                        interpolate2fine(q, aux, child[0], child[1], c, self.phys)
                    new[ck] = child
            elif not any(k in fam for fam in merges):
                new[k] = [q, aux]
        for fam in merges:
            l, I, J = fam[0]
            pk = (l - 1, I >> 1, J >> 1)
            parent = self.new_patch(pk, False)
            for c, ck in enumerate(fam):
                average2coarse(parent[0], parent[1], self.leaves[ck][0], self.leaves[ck][1], c,
                               self.phys)
            new[pk] = parent
        changed = bool(split) or bool(merges)
        self.leaves = new
        return changed

    def regrid(self, t):
        self.ghost_fill(t)
        refine, fams = self._tags(t, 0)
        split = {k for k, v in refine.items() if v}
        self._balance(split)
        merges = []
        for fam, c in fams:
            if c and not any(f in split for f in fam) and \
                    self._can_merge(fam[0][0], fam[0][1] >> 1, fam[0][2] >> 1, split):
                merges.append(fam)
        self.regrids += 1
        return self._apply(split, merges, False)

    def init(self):
        self.leaves = {}
        for J in range(self.npy(self.lmin)):
            for I in range(self.npx(self.lmin)):
                k = (self.lmin, I, J)
                self.leaves[k] = self.new_patch(k, True)
        for _ in range(self.lmin, self.lmax):
            refine, _ = self._tags(0.0, 1)
            split = {k for k, v in refine.items() if v}
            self._balance(split)
            if not self._apply(split, [], True):
                break

    # ---- stepping -------------------------------------------------------
    def step(self, t, dt):
        """Ghost fill at t and one update of every leaf; returns max CFL."""
        self.ghost_fill(t)
        keys = self.canonical()
        q = np.stack([self.leaves[k][0] for k in keys])
        aux = np.stack([self.leaves[k][1] for k in keys])
        dx = np.array([self.dx(k[0]) for k in keys])
        dy = np.array([self.dy(k[0]) for k in keys])
        cfl = level_update(q, aux, dx, dy, t, dt, self.phys)
        for n, k in enumerate(keys):
            self.leaves[k][0][...] = q[n]
        return cfl

    def snapshot(self):
        return {k: v[0].copy() for k, v in self.leaves.items()}

    def restore(self, snap):
        for k, q in snap.items():
            self.leaves[k][0][...] = q

    def run(self, t_final, nout, initial_dt, desired_cfl, max_cfl, max_steps=0):
        """outstyle 1 (src/fc2d_geoclaw/fc2d_geoclaw_run.c:190-395), variable dt,
        advance-one-step, no subcycling; returns the accepted dt list."""
        level_factor = float(1 << (self.lmax - self.lmin))
        dt_outer = t_final / nout
        t_curr = self.t
        dt_minlevel = initial_dt
        taken = 0
        dts = []
        if not self.out_started:
            if self.frames:
                self.write_frame(self.out_dir, self.next_frame)
                self.next_frame += 1
            self.sample_gauges(t_curr)
            self.out_started = True
        for _ in range(nout):
            tend = t_curr + dt_outer
            while t_curr < tend:
                if max_steps and taken >= max_steps:
                    self.t, self.dt = t_curr, dt_minlevel
                    self.flush_gauges()
                    return dts
                dt_step = dt_minlevel if self.subcycle else dt_minlevel / level_factor
                tol = 1e-2 * dt_step
                took_small = False
                small_step = tend - (t_curr + dt_step)
                if small_step < tol:
                    dt_step = tend - t_curr
                    if small_step < 0:
                        took_small = True
                snap = self.snapshot()
                if self.subcycle:
                    cfl, cu = self.step_subcycled(t_curr, dt_step)
                else:
                    cfl, cu = self.step(t_curr, dt_step), len(self.leaves) * self.m * self.m
                taken += 1
                self.max_cfl_seen = max(self.max_cfl_seen, cfl)
                if cfl > max_cfl:
                    self.restore(snap)
                    dt_minlevel = dt_minlevel * desired_cfl / cfl
                    self.rejects += 1
                    continue
                self.steps += 1
                self.cell_updates += cu
                t_curr += dt_step
                dts.append(dt_step)
                dt_new = dt_minlevel * desired_cfl / cfl if cfl > 0.0 else float("inf")
                if not took_small:
                    dt_minlevel = dt_new
                self.t = t_curr
                self.sample_gauges(t_curr)
                if self.regrid_interval > 0 and self.steps % self.regrid_interval == 0:
                    self.regrid(t_curr)
            if self.frames:
                self.flush_gauges()
                self.write_frame(self.out_dir, self.next_frame)
                self.next_frame += 1
        self.t, self.dt = t_curr, dt_minlevel
        self.flush_gauges()
        return dts

    # ---- output -----------------------------------------------------------
    def set_output(self, out_dir, frames=True):
        self.out_dir, self.frames = out_dir, bool(frames)

    def set_gauges(self, gauges):
        """gauges: [(id, x, y, t1, t2, min_time_increment)]; writes the headers."""
        self.gauges = []
        for gid, x, y, t1, t2, incr in gauges:
            self.gauges.append(dict(id=gid, x=x, y=y, t1=t1, t2=t2, incr=incr, last=-np.inf,
                                    rows=[]))
            with open(os.path.join(self.out_dir, "gauge%05d.txt" % gid), "w") as f:
                f.write(fout.gauge_header(gid, x, y))

    def frame_arrays(self):
        keys = self.canonical()
        order, trees = fout.p4est_order(keys, self.nbx, self.nby, self.lmax)
        ks = [keys[n] for n in order]
        q = np.stack([self.leaves[k][0] for k in ks])
        aux = np.stack([self.leaves[k][1] for k in ks])
        org = [self.origin(*k) for k in ks]
        return (q, aux, [k[0] for k in ks], [trees[n] for n in order], [o[0] for o in org],
                [o[1] for o in org], [self.dx(k[0]) for k in ks], [self.dy(k[0]) for k in ks])

    def write_frame(self, out_dir, iframe):
        fout.write_frame(out_dir, iframe, self.t, *self.frame_arrays())

    def _gauge_leaf(self, g):
        """(key, ii, jj, xoff, yoff) of the leaf holding gauge g, or None."""
        L, m = self.lmax, self.m
        ux = (g["x"] - self.x0) / (m * self.dx(L))
        uy = (g["y"] - self.y0) / (m * self.dy(L))
        if not (ux >= 0.0 and uy >= 0.0) or ux > self.npx(L) or uy > self.npy(L):
            return None
        IF = min(int(np.floor(ux)), self.npx(L) - 1)
        JF = min(int(np.floor(uy)), self.npy(L) - 1)
        key = self.containing(L, IF, JF)
        if key is None:
            return None
        xl, yl = self.origin(*key)
        return (key,) + fout.gauge_cell(m, xl, yl, self.dx(key[0]), self.dy(key[0]), g["x"], g["y"])

    def sample_gauges(self, t):
        """One record per gauge whose window holds t, after exchanging ghost
        cells at t when a stencil reaches them."""
        if not self.gauges:
            return
        place = [self._gauge_leaf(g) for g in self.gauges]
        if any(p is not None and (p[1] >= self.m or p[2] >= self.m)
               for p in place) and any(p is not None and g["t1"] <= t <= g["t2"]
                                       for p, g in zip(place, self.gauges)):
            self.ghost_fill(t)
        drytol = params(self.phys).dry_tolerance
        for p, g in zip(place, self.gauges):
            if p is None or not (g["t1"] <= t <= g["t2"] and t >= g["last"] + g["incr"]
                                 and t > g["last"]):
                continue
            key, ii, jj, xo, yo = p
            q, aux = self.leaves[key]
            g["rows"].append((key[0], t) + fout.sample_gauge(q, aux, ii, jj, xo, yo, drytol))
            g["last"] = t

    def flush_gauges(self):
        for g in self.gauges:
            if g["rows"]:
                with open(os.path.join(self.out_dir, "gauge%05d.txt" % g["id"]), "a") as f:
                    f.write(fout.gauge_rows(g["rows"]))
                g["rows"] = []

    def patches(self):
        return np.array(self.canonical(), np.int32).reshape(-1, 3)

    def download(self):
        return np.stack([self.leaves[k][0] for k in self.canonical()])

    def download_aux(self):
        return np.stack([self.leaves[k][1] for k in self.canonical()])

    def upload(self, q):
        for n, k in enumerate(self.canonical()):
            self.leaves[k][0][...] = q[n]

    def adopt(self, patches, q):
        """Take another forest's leaves and states: patches (n, 3) of (level,
        I, J) in canonical order with q (n, my+4, mx+4, 3); each leaf's aux
        comes from this forest's own raster pyramid. Lets a checker restart
        this forest from the state of the forest it checks."""
        self.leaves = {}
        for n, p in enumerate(np.asarray(patches).reshape(-1, 3)):
            key = (int(p[0]), int(p[1]), int(p[2]))
            self.leaves[key] = [np.array(q[n], np.float64), self.new_patch(key, False)[1]]
