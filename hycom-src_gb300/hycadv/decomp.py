"""One basin split over ranks: 2-D blocks with halos exchanged between
neighbours, the form of the reference's MPI build (mod_xc_mp.h:4664-4987,
xctilr over tiles) for a basin too large for one GPU.

Each rank owns a block of the interior with an nbdy-wide halo and runs the
advection on it in the library's external-halo mode (a context created with
nreg = HYC_NREG_EXTERNAL, whose xctilr leaves halos alone).  Before each
tsadvc the caller fills the halos of the fields tsadvc refreshes with
:func:`Decomp.exchange`: first east-west (every row), then north-south
(every column, so the corners come from the diagonal neighbour through the
first phase).  At the basin's own edges the fill is xctilr's: a periodic
copy in x when the basin is periodic, zero (vland) otherwise.  The interior
results then equal a single-domain run bit for bit: every cell is computed
from the same values in the same order.

The exchange runs over torch.distributed point-to-point (gloo on CPU,
NCCL between GPUs; each message lands in the receiver's own buffer), or
between in-process tiles (:meth:`Decomp.exchange_tiles`) for tests on one
device.

Conservation sums use the reference's reproducible xcsum
(mod_xc_mp.h:3353-3533): partial row sums over strips 2*nbdy+1 columns
wide, each formed on the block that owns the strip's centre (from its
halo), then added in global column order, and the rows in global row
order -- so a decomposed basin's sum equals the single-domain sum bit for
bit, whatever the block layout (:meth:`Decomp.xcsum`,
:meth:`Decomp.xcsum_tiles`).
"""
from __future__ import annotations

import numpy as np


def _split(n: int, p: int) -> list[tuple[int, int]]:
    """1-based inclusive ranges of n cells over p parts, sizes differ by <= 1."""
    base, extra = divmod(n, p)
    out, a = [], 1
    for q in range(p):
        m = base + (1 if q < extra else 0)
        out.append((a, a + m - 1))
        a += m
    return out


class Decomp:
    def __init__(self, nx: int, ny: int, nbdy: int, px: int, py: int, periodic: bool):
        if px < 1 or py < 1 or px > nx or py > ny:
            raise ValueError("bad process grid")
        self.nx, self.ny, self.nbdy, self.px, self.py, self.periodic = nx, ny, nbdy, px, py, periodic
        self.xs = _split(nx, px)
        self.ys = _split(ny, py)

    @property
    def size(self) -> int:
        return self.px * self.py

    def coords(self, r: int) -> tuple[int, int]:
        return r % self.px, r // self.px

    def rank_of(self, pi: int, pj: int) -> int:
        return pj * self.px + pi

    def extent(self, r: int) -> tuple[int, int, int, int]:
        """(i0, i1, j0, j1): the block's interior, 1-based inclusive basin indices."""
        pi, pj = self.coords(r)
        return self.xs[pi][0], self.xs[pi][1], self.ys[pj][0], self.ys[pj][1]

    def dims(self, r: int) -> tuple[int, int]:
        i0, i1, j0, j1 = self.extent(r)
        return i1 - i0 + 1, j1 - j0 + 1

    def neighbour(self, r: int, d: str):
        """Rank west/east/south/north of r, or None at a closed basin edge."""
        pi, pj = self.coords(r)
        if d in ("west", "east"):
            qi = pi - 1 if d == "west" else pi + 1
            if 0 <= qi < self.px:
                return self.rank_of(qi, pj)
            return self.rank_of(qi % self.px, pj) if self.periodic else None
        qj = pj - 1 if d == "south" else pj + 1
        return self.rank_of(pi, qj) if 0 <= qj < self.py else None

    def window(self, a, r: int):
        """The block of rank r with its halo, from a basin array (..., ld2, ld1)
        in the reference layout (a copy)."""
        i0, i1, j0, j1 = self.extent(r)
        nb = self.nbdy
        # python index of basin cell (i, j) is (j + nb - 1, i + nb - 1)
        sub = a[..., j0 - 1:j1 + 2 * nb, i0 - 1:i1 + 2 * nb]
        return sub.copy() if isinstance(sub, np.ndarray) else sub.clone()

    def interior(self, a_local, r: int):
        nx, ny = self.dims(r)
        nb = self.nbdy
        return a_local[..., nb:nb + ny, nb:nb + nx]

    def insert(self, a, a_local, r: int):
        """Write rank r's interior back into the basin array a."""
        i0, i1, j0, j1 = self.extent(r)
        nb = self.nbdy
        a[..., j0 + nb - 1:j1 + nb, i0 + nb - 1:i1 + nb] = self.interior(a_local, r)

    # -- strips (python index ranges of a local array) -----------------------
    def _cols(self, r: int, w: int):
        nx, _ = self.dims(r)
        nb = self.nbdy
        return {"west_in": slice(nb, nb + w), "east_in": slice(nb + nx - w, nb + nx),
                "west_halo": slice(nb - w, nb), "east_halo": slice(nb + nx, nb + nx + w)}

    def _rows(self, r: int, w: int):
        _, ny = self.dims(r)
        nb = self.nbdy
        return {"south_in": slice(nb, nb + w), "north_in": slice(nb + ny - w, nb + ny),
                "south_halo": slice(nb - w, nb), "north_halo": slice(nb + ny, nb + ny + w)}

    def _check_width(self, w: int):
        if w < 1 or w > self.nbdy:
            raise ValueError("halo width must be in 1..nbdy")
        if min(b - a + 1 for a, b in self.xs) < w or min(b - a + 1 for a, b in self.ys) < w:
            raise ValueError("every block must be at least the halo width wide")

    # -- in-process exchange (tests on one device) --------------------------
    def exchange_tiles(self, tiles: list, w: int):
        """Fill the w-wide halos of every rank's local array (tiles[r], numpy or
        torch, (..., ld2, ld1)) from its neighbours, as exchange() does."""
        self._check_width(w)
        for phase in ("x", "y"):
            new = []
            for r, t in enumerate(tiles):
                fills = {}
                dirs = ("west", "east") if phase == "x" else ("south", "north")
                for d in dirs:
                    q = self.neighbour(r, d)
                    opp = {"west": "east", "east": "west", "south": "north", "north": "south"}[d]
                    if q is None:
                        fills[d] = None
                    elif phase == "x":
                        fills[d] = tiles[q][..., :, self._cols(q, w)[opp + "_in"]]
                    else:
                        fills[d] = tiles[q][..., self._rows(q, w)[opp + "_in"], :]
                    fills[d] = None if fills[d] is None else (
                        fills[d].copy() if isinstance(fills[d], np.ndarray) else fills[d].clone())
                new.append(fills)
            for r, t in enumerate(tiles):
                self._apply(t, r, new[r], w, phase)

    def _apply(self, t, r: int, fills: dict, w: int, phase: str):
        if phase == "x":
            c = self._cols(r, w)
            for d in ("west", "east"):
                v = fills[d]
                if v is None:
                    t[..., :, c[d + "_halo"]] = 0.0
                else:
                    t[..., :, c[d + "_halo"]] = v
        else:
            rw = self._rows(r, w)
            for d in ("south", "north"):
                v = fills[d]
                if v is None:
                    t[..., rw[d + "_halo"], :] = 0.0
                else:
                    t[..., rw[d + "_halo"], :] = v

    # -- distributed exchange ----------------------------------------------
    def exchange(self, t, w: int, dist, rank: int):
        """Fill the w-wide halos of this rank's local torch tensor t (..., ld2,
        ld1) from its neighbours over torch.distributed point-to-point
        (every rank calls it for the same field, in the same order)."""
        import torch

        self._check_width(w)
        opp = {"west": "east", "east": "west", "south": "north", "north": "south"}
        tag = {"west": 1, "east": 2, "south": 3, "north": 4}
        for phase, dirs in (("x", ("west", "east")), ("y", ("south", "north"))):
            sl = self._cols(rank, w) if phase == "x" else self._rows(rank, w)
            fills, reqs, bufs, keep = {}, [], {}, []
            for d in dirs:
                q = self.neighbour(rank, d)
                if q is None:
                    fills[d] = None
                    continue
                out = t[..., :, sl[d + "_in"]] if phase == "x" else t[..., sl[d + "_in"], :]
                if q == rank:  # periodic with one block across: a local copy
                    fills[opp[d]] = out.clone()
                    continue
                snd = out.contiguous()
                inb = torch.empty_like(snd)
                bufs[d] = inb
                keep.append(snd)
                # my d-side strip goes to neighbour q as its opposite-side halo;
                # its opposite-side strip arrives from q into my d-side halo
                reqs.append(dist.isend(snd, q, tag=tag[opp[d]]))
                reqs.append(dist.irecv(inb, q, tag=tag[d]))
            for rq in reqs:
                rq.wait()
            for d, b in bufs.items():
                fills[d] = b
            self._apply(t, rank, fills, w, phase)

    # -- reproducible sums (xcsum) ------------------------------------------
    def _centres(self):
        """Global centres of the partial-sum strips (mod_xc_mp.h:2915)."""
        return list(range(1 + self.nbdy, self.nx + self.nbdy + 1, 2 * self.nbdy + 1))

    def _partials(self, a_local, mask_local, r: int) -> dict:
        """Rank r's partial row sums {(j, l): sum} over the strips whose
        centre it owns (its interior, or for the last block of a row of
        blocks the nbdy columns east of it, mod_xc_mp.h:2895-2936), summed in
        column order from its window (halo included, mod_xc_mp.h:3410-3424)."""
        nb = self.nbdy
        i0, i1, j0, j1 = self.extent(r)
        last = self.coords(r)[0] == self.px - 1
        a = np.asarray(a_local, dtype=np.float64)
        m = np.asarray(mask_local)
        out = {}
        for l, c in enumerate(self._centres()):
            if not (i0 <= c <= i1 or (last and i1 < c <= i1 + nb)):
                continue
            lo, hi = max(c - nb, 1), min(c + nb, self.nx)
            cols = range(lo - i0 + nb, hi - i0 + nb + 1)  # local index of global column i: i - i0 + nb
            for j in range(j0, j1 + 1):
                row = j - j0 + nb
                s = 0.0
                for q in cols:
                    if m[row, q] == 1:
                        s = s + float(a[row, q])
                out[(j, l)] = s
        return out

    def _total(self, parts) -> float:
        allp = {}
        for p in parts:
            allp.update(p)
        total = 0.0
        for j in range(1, self.ny + 1):
            s8 = 0.0
            for l in range(len(self._centres())):
                s8 = s8 + allp[(j, l)]
            total = total + s8
        return total

    def xcsum_tiles(self, tiles: list, masks: list) -> float:
        """xcsum of a field held as every rank's local array (halos filled)."""
        return self._total([self._partials(t, m, r) for r, (t, m) in enumerate(zip(tiles, masks))])

    def xcsum(self, a_local, mask_local, dist, rank: int) -> float:
        """xcsum over all ranks (every rank calls it; all get the same
        value).  a_local (ld2, ld1) needs its halo filled first (the
        reference refreshes it with xctilr before summing)."""
        parts = [None] * self.size
        dist.all_gather_object(parts, self._partials(a_local, mask_local, rank))
        return self._total(parts)
