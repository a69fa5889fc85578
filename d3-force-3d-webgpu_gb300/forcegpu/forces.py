"""The force objects of d3-force-3d, as descriptors for the GPU engine.

Same constructors, accessors and defaults as the reference's src/*.js forces; each evaluates its
accessors per node / per link in initialize() (bumping `version`, as the reference does) and
describes itself with gpu(), the dictionary the engine turns into an fl_force_desc. The physics
runs only on the GPU: a force object is not callable on the CPU.

Nodes are dicts with x, y, z, vx, vy, vz, fx, fy, fz (None for unset), as the reference's node
objects; links are dicts with source and target (a node, or an id resolved by initialize()).
"""
from __future__ import annotations

import math

_UNSET = object()


def constant(x):
    """src/constant.js: a function that always returns x."""
    return lambda *args: x


def _num(v):
    """+v of JavaScript for a numeric accessor result (None -> NaN)."""
    if v is None:
        return math.nan
    try:
        return float(v)
    except (TypeError, ValueError):
        return math.nan


def _accessor(value):
    return value if callable(value) else constant(_num(value))


class Force:
    """Base: name, version, initialize(nodes, random, nDim), gpu()."""

    type = None

    def __init__(self):
        self._nodes = None
        self._version = 0

    def __call__(self, alpha=None):
        raise RuntimeError("%s runs on the GPU engine only (forceSimulationGPU)" % type(self).__name__)

    def initialize(self, nodes, random=None, nDim=2):
        self._nodes = nodes
        self._random = random
        self._nDim = nDim if nDim in (1, 2, 3) else 2
        self._initialize()

    def _initialize(self):
        pass

    def gpu(self):
        raise NotImplementedError


class ManyBody(Force):
    """src/manyBody.js: strength -30, distanceMin 1, distanceMax inf, theta 0.9."""

    type = "manyBody"

    def __init__(self):
        super().__init__()
        self._strength = constant(-30.0)
        self._strengths = []
        self._distanceMin2 = 1.0
        self._distanceMax2 = math.inf
        self._theta2 = 0.81

    def _initialize(self):
        if self._nodes is None:
            return
        nodes = self._nodes
        s = [0.0] * len(nodes)
        for i, node in enumerate(nodes):
            s[node.get("index", i)] = _num(self._strength(node, i, nodes))
        self._strengths = s
        self._version += 1

    def strength(self, _=_UNSET):
        if _ is _UNSET:
            return self._strength
        self._strength = _accessor(_)
        self._initialize()
        return self

    def distanceMin(self, _=_UNSET):
        if _ is _UNSET:
            return math.sqrt(self._distanceMin2)
        self._distanceMin2 = float(_) * float(_)
        return self

    def distanceMax(self, _=_UNSET):
        if _ is _UNSET:
            return math.sqrt(self._distanceMax2)
        self._distanceMax2 = float(_) * float(_)
        return self

    def theta(self, _=_UNSET):
        if _ is _UNSET:
            return math.sqrt(self._theta2)
        self._theta2 = float(_) * float(_)
        return self

    def gpu(self):
        return {"type": "manyBody", "version": self._version, "strengths": self._strengths,
                "distanceMin2": self._distanceMin2, "distanceMax2": self._distanceMax2,
                "theta2": self._theta2}


class Link(Force):
    """src/link.js: distance 30, strength 1 / min(count), bias count[s] / (count[s] + count[t])."""

    type = "link"

    def __init__(self, links=None):
        super().__init__()
        self._links = list(links) if links is not None else []
        self._id = lambda d, *a: d.get("index")
        self._strength = self._default_strength
        self._distance = constant(30.0)
        self._iterations = 1
        self._count = []
        self._bias = []
        self._strengths = []
        self._distances = []

    def _default_strength(self, link, *args):
        return 1.0 / min(self._count[link["source"]["index"]], self._count[link["target"]["index"]])

    def _initialize(self):
        if self._nodes is None:
            return
        nodes, links = self._nodes, self._links
        by_id = {}
        for i, d in enumerate(nodes):
            by_id[self._id(d, i, nodes)] = d
        count = [0] * len(nodes)
        for i, link in enumerate(links):
            link["index"] = i
            for end in ("source", "target"):
                if not isinstance(link[end], dict):
                    key = link[end]
                    if key not in by_id:
                        raise KeyError("node not found: %r" % (key,))
                    link[end] = by_id[key]
            count[link["source"]["index"]] += 1
            count[link["target"]["index"]] += 1
        self._count = count
        self._bias = [count[l["source"]["index"]] / (count[l["source"]["index"]] + count[l["target"]["index"]])
                      for l in links]
        self._strengths = [0.0] * len(links)
        self._distances = [0.0] * len(links)
        self._initialize_strength()
        self._initialize_distance()

    def _initialize_strength(self):
        if self._nodes is None:
            return
        links = self._links
        self._strengths = [_num(self._strength(l, i, links)) for i, l in enumerate(links)]
        self._version += 1

    def _initialize_distance(self):
        if self._nodes is None:
            return
        links = self._links
        self._distances = [_num(self._distance(l, i, links)) for i, l in enumerate(links)]
        self._version += 1

    def links(self, _=_UNSET):
        if _ is _UNSET:
            return self._links
        self._links = list(_)
        self._initialize()
        return self

    def id(self, _=_UNSET):
        if _ is _UNSET:
            return self._id
        self._id = _
        return self

    def iterations(self, _=_UNSET):
        if _ is _UNSET:
            return self._iterations
        self._iterations = int(_)
        return self

    def strength(self, _=_UNSET):
        if _ is _UNSET:
            return self._strength
        self._strength = _accessor(_)
        self._initialize_strength()
        return self

    def distance(self, _=_UNSET):
        if _ is _UNSET:
            return self._distance
        self._distance = _accessor(_)
        self._initialize_distance()
        return self

    def gpu(self):
        return {"type": "link", "version": self._version, "links": self._links,
                "iterations": self._iterations, "strengths": self._strengths,
                "distances": self._distances, "bias": self._bias}


class Collide(Force):
    """src/collide.js: radius 1, strength 1, iterations 1."""

    type = "collide"

    def __init__(self, radius=None):
        super().__init__()
        self._radius = radius if callable(radius) else constant(1.0 if radius is None else _num(radius))
        self._strength = 1.0
        self._iterations = 1
        self._radii = []

    def _initialize(self):
        if self._nodes is None:
            return
        nodes = self._nodes
        r = [0.0] * len(nodes)
        for i, node in enumerate(nodes):
            r[node.get("index", i)] = _num(self._radius(node, i, nodes))
        self._radii = r
        self._version += 1

    def iterations(self, _=_UNSET):
        if _ is _UNSET:
            return self._iterations
        self._iterations = int(_)
        return self

    def strength(self, _=_UNSET):
        if _ is _UNSET:
            return self._strength
        self._strength = float(_)
        return self

    def radius(self, _=_UNSET):
        if _ is _UNSET:
            return self._radius
        self._radius = _accessor(_)
        self._initialize()
        return self

    def gpu(self):
        return {"type": "collide", "version": self._version, "radii": self._radii,
                "strength": self._strength, "iterations": self._iterations}


class Center(Force):
    """src/center.js: shift every node so that the mean sits at (x, y, z); strength 1."""

    type = "center"

    def __init__(self, x=None, y=None, z=None):
        super().__init__()
        self._x = 0.0 if x is None else float(x)
        self._y = 0.0 if y is None else float(y)
        self._z = 0.0 if z is None else float(z)
        self._strength = 1.0

    def x(self, _=_UNSET):
        if _ is _UNSET:
            return self._x
        self._x = float(_)
        return self

    def y(self, _=_UNSET):
        if _ is _UNSET:
            return self._y
        self._y = float(_)
        return self

    def z(self, _=_UNSET):
        if _ is _UNSET:
            return self._z
        self._z = float(_)
        return self

    def strength(self, _=_UNSET):
        if _ is _UNSET:
            return self._strength
        self._strength = float(_)
        return self

    def gpu(self):
        return {"type": "center", "version": 0, "x": self._x, "y": self._y, "z": self._z,
                "strength": self._strength}


class Radial(Force):
    """src/radial.js: pull every node towards the sphere of radius r_i around (x, y, z)."""

    type = "radial"

    def __init__(self, radius=None, x=None, y=None, z=None):
        super().__init__()
        self._radius = _accessor(radius)
        self._strength = constant(0.1)
        self._x = 0.0 if x is None else float(x)
        self._y = 0.0 if y is None else float(y)
        self._z = 0.0 if z is None else float(z)
        self._radiuses = []
        self._strengths = []

    def _initialize(self):
        if self._nodes is None:
            return
        nodes = self._nodes
        self._radiuses = [_num(self._radius(d, i, nodes)) for i, d in enumerate(nodes)]
        self._strengths = [0.0 if math.isnan(self._radiuses[i]) else _num(self._strength(d, i, nodes))
                           for i, d in enumerate(nodes)]
        self._version += 1

    def strength(self, _=_UNSET):
        if _ is _UNSET:
            return self._strength
        self._strength = _accessor(_)
        self._initialize()
        return self

    def radius(self, _=_UNSET):
        if _ is _UNSET:
            return self._radius
        self._radius = _accessor(_)
        self._initialize()
        return self

    def x(self, _=_UNSET):
        if _ is _UNSET:
            return self._x
        self._x = float(_)
        return self

    def y(self, _=_UNSET):
        if _ is _UNSET:
            return self._y
        self._y = float(_)
        return self

    def z(self, _=_UNSET):
        if _ is _UNSET:
            return self._z
        self._z = float(_)
        return self

    def gpu(self):
        return {"type": "radial", "version": self._version, "radiuses": self._radiuses,
                "strengths": self._strengths, "x": self._x, "y": self._y, "z": self._z}


class Position(Force):
    """src/x.js, y.js, z.js: v[axis] += (target_i - p[axis]) * strength_i * alpha."""

    type = "position"
    axis = 0
    _name = "x"

    def __init__(self, target=None):
        super().__init__()
        self._target = target if callable(target) else constant(0.0 if target is None else _num(target))
        self._strength = constant(0.1)
        self._targets = []
        self._strengths = []

    def _initialize(self):
        if self._nodes is None:
            return
        nodes = self._nodes
        self._targets = [_num(self._target(d, i, nodes)) for i, d in enumerate(nodes)]
        self._strengths = [0.0 if math.isnan(self._targets[i]) else _num(self._strength(d, i, nodes))
                           for i, d in enumerate(nodes)]
        self._version += 1

    def initialize(self, nodes, random=None, nDim=2):
        self._nodes = nodes
        self._initialize()

    def strength(self, _=_UNSET):
        if _ is _UNSET:
            return self._strength
        self._strength = _accessor(_)
        self._initialize()
        return self

    def _goal(self, _=_UNSET):
        if _ is _UNSET:
            return self._target
        self._target = _accessor(_)
        self._initialize()
        return self

    def gpu(self):
        return {"type": "position", "axis": self.axis, "version": self._version,
                "targets": self._targets, "strengths": self._strengths}


class PositionX(Position):
    axis = 0

    def x(self, _=_UNSET):
        return self._goal(_)


class PositionY(Position):
    axis = 1

    def y(self, _=_UNSET):
        return self._goal(_)


class PositionZ(Position):
    axis = 2

    def z(self, _=_UNSET):
        return self._goal(_)


def forceManyBody():
    return ManyBody()


def forceLink(links=None):
    return Link(links)


def forceCollide(radius=None):
    return Collide(radius)


def forceCenter(x=None, y=None, z=None):
    return Center(x, y, z)


def forceRadial(radius=None, x=None, y=None, z=None):
    return Radial(radius, x, y, z)


def forceX(x=None):
    return PositionX(x)


def forceY(y=None):
    return PositionY(y)


def forceZ(z=None):
    return PositionZ(z)
