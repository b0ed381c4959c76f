"""Geometric regions used to populate solids and define groups (host setup).

Restates src/region_block.cpp, src/region_cylinder.cpp and
src/region_sphere.cpp: ``inside`` is inclusive of the surface, ``limits`` is
the bounding box, ``match`` honours the ``exterior`` option
(src/region.cpp:65-74).  Block regions extend the domain box when they reach
past it (src/region_block.cpp:45-120).
"""
from __future__ import annotations

import numpy as np

BIG = 1.0e20  # src/region_block.cpp / src/region_cylinder.cpp: #define BIG


def _inf_value(tok, sign, have_regions):
    if isinstance(tok, str) and tok.lstrip("+-") in ("INF", "EDGE"):
        if not have_regions:
            raise ValueError("Cannot use region INF or EDGE when box does not exist.")
        return sign * BIG
    return float(tok)


class Region:
    interior = True

    def match(self, x):
        x = np.atleast_2d(x)
        return self.inside(x) if self.interior else ~self.inside(x)


class Block(Region):
    def __init__(self, args, dim, boxlo, boxhi, have_regions):
        need = {1: 2, 2: 4, 3: 6}[dim]
        if len(args) < need:
            raise ValueError("Error: region command not enough arguments.")
        self.lo, self.hi = np.zeros(3), np.zeros(3)
        for d in range(dim):
            lo = _inf_value(args[2 * d], -1, have_regions)
            hi = _inf_value(args[2 * d + 1], +1, have_regions)
            if abs(lo) != BIG and boxlo[d] > lo:
                boxlo[d] = lo
            if abs(hi) != BIG and boxhi[d] < hi:
                boxhi[d] = hi
            self.lo[d], self.hi[d] = lo, hi
        if np.any(self.lo > self.hi):
            raise ValueError("Illegal region block command.")
        self.interior = "exterior" not in [str(a) for a in args[need:]]

    def inside(self, x):
        x = np.atleast_2d(x)
        return np.all((x >= self.lo) & (x <= self.hi), axis=1)

    def limits(self):
        return [self.lo[0], self.hi[0], self.lo[1], self.hi[1], self.lo[2], self.hi[2]]


class Cylinder(Region):
    def __init__(self, args, dim, boxlo, boxhi, have_regions):
        if dim == 3:
            if len(args) < 6:
                raise ValueError("Error: not enough arguments.")
            self.axis = str(args[0])
            if self.axis not in ("x", "y", "z"):
                raise ValueError("region cylinder axis not understood")
            self.c1, self.c2, self.R = float(args[1]), float(args[2]), float(args[3])
            self.lo = _inf_value(args[4], -1, have_regions)
            self.hi = _inf_value(args[5], +1, have_regions)
            extra = args[6:]
        else:
            if len(args) < 3:
                raise ValueError("Error: not enough arguments.")
            self.axis = "z"
            self.c1, self.c2, self.R = float(args[0]), float(args[1]), float(args[2])
            self.lo = self.hi = 0.0
            extra = args[3:]
        if self.lo > self.hi:
            raise ValueError("Illegal region cylinder command: low is higher than high.")
        self.RSq = self.R * self.R
        self.interior = "exterior" not in [str(a) for a in extra]

    def _split(self, x):
        ax = "xyz".index(self.axis)
        o = [d for d in range(3) if d != ax]
        return x[:, ax], x[:, o[0]], x[:, o[1]]

    def inside(self, x):
        x = np.atleast_2d(x)
        a, p, q = self._split(x)
        dSq = (p - self.c1) ** 2 + (q - self.c2) ** 2
        return (a >= self.lo) & (a <= self.hi) & (dSq <= self.RSq)

    def limits(self):
        c1lo, c1hi, c2lo, c2hi = self.c1 - self.R, self.c1 + self.R, self.c2 - self.R, self.c2 + self.R
        if self.axis == "x":
            return [self.lo, self.hi, c1lo, c1hi, c2lo, c2hi]
        if self.axis == "y":
            return [c1lo, c1hi, self.lo, self.hi, c2lo, c2hi]
        return [c1lo, c1hi, c2lo, c2hi, self.lo, self.hi]


class Sphere(Region):
    def __init__(self, args, dim, boxlo, boxhi, have_regions):
        self.c = np.zeros(3)
        for d in range(3):
            self.c[d] = float(args[d])
        self.R = float(args[3])
        self.interior = "exterior" not in [str(a) for a in args[4:]]

    def inside(self, x):
        x = np.atleast_2d(x)
        return np.sum((x - self.c) ** 2, axis=1) <= self.R * self.R

    def limits(self):
        return [self.c[0] - self.R, self.c[0] + self.R, self.c[1] - self.R, self.c[1] + self.R,
                self.c[2] - self.R, self.c[2] + self.R]


def make_region(kind, args, dim, boxlo, boxhi, nregions):
    cls = {"block": Block, "cylinder": Cylinder, "sphere": Sphere}.get(kind)
    if cls is None:
        raise ValueError(f"region style {kind} is not supported by the GPU path's host setup")
    return cls(list(args), dim, boxlo, boxhi, nregions > 0)
