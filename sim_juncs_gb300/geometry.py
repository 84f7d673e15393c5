"""CSG objects of the CGS scene language, flattened into the postfix
programs the device rasteriser evaluates (``sj_csg_node``).

The primitives restate the constructors and ``in()`` of src/cgs.cpp:
``Box`` (src/cgs.cpp:41-70), ``Sphere`` (:23-39), ``Plane`` (:76-99),
``Cylinder`` (:103-120) and ``composite_object`` (:403-449), so that a scene
built here answers ``in(r)`` exactly as the reference's objects do.  Vector
arithmetic follows src/geometry.hpp's operation order (Python floats are
IEEE doubles, so the same sequence gives the same bits).
"""
import math

from . import _abi

IDENTITY = (1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0)


def _matmul(a, b):
    # matrix::operator* (src/geometry.hpp:88-99): sum over k starting from 0
    out = []
    for i in range(3):
        for j in range(3):
            s = 0.0
            for k in range(3):
                s += a[3 * i + k] * b[3 * k + j]
            out.append(s)
    return tuple(out)


def _cross(a, b):
    return (a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0])


def _dot(a, b):
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]


def _normalize(v):
    s = 0.0
    for x in v:
        s += x * x
    n = math.sqrt(s)
    return tuple(x / n for x in v)


def rotation(theta, axis):
    """Rotation matrix about `axis` by `theta` (row-major 3x3)."""
    ax = _normalize(axis)
    c, s = math.cos(theta), math.sin(theta)
    x, y, z = ax
    return (c + x * x * (1 - c), x * y * (1 - c) - z * s, x * z * (1 - c) + y * s,
            y * x * (1 - c) + z * s, c + y * y * (1 - c), y * z * (1 - c) - x * s,
            z * x * (1 - c) - y * s, z * y * (1 - c) + x * s, c + z * z * (1 - c))


class Obj:
    invert = 0
    trans = IDENTITY

    def inverted(self):
        """Return this object with its inclusion inverted (CGS Complement)."""
        self.invert ^= 1
        return self


class Box(Obj):
    """box(p1, p2): |trans*(r - center)|_inf <= offset, faces inclusive."""

    def __init__(self, p1, p2, invert=0, trans=IDENTITY):
        off = [(p2[a] - p1[a]) / 2 for a in range(3)]
        self.center = tuple(p1[a] + off[a] for a in range(3))
        self.offset = tuple(-o if o < 0 else o for o in off)
        self.invert = invert
        self.trans = trans


class Sphere(Obj):
    def __init__(self, center, rad, invert=0, trans=IDENTITY):
        self.center = tuple(center)
        self.rad = float(rad)
        self.invert = invert
        self.trans = trans


class Cylinder(Obj):
    """cylinder(center, height, r1, r2): a cone frustum along the local z axis."""

    def __init__(self, center, height, r1, r2, invert=0, trans=IDENTITY):
        self.center = tuple(center)
        self.height = float(height)
        self.r1_sq = r1 * r1
        self.r2_sq = r2 * r2
        self.invert = invert
        self.trans = trans


class Plane(Obj):
    """plane: points with dot(r, normal) <= offset.

    Plane(normal, offset) or Plane(p1, p2, p3) with normal (p2-p1)x(p3-p1).
    Like the reference, inversion only negates the offset at construction;
    a later Complement/Difference leaves a plane unchanged.
    """

    def __init__(self, a, b, c=None, invert=0):
        if c is None:
            self.normal = _normalize(tuple(a))
            self.offset = -float(b) if invert else float(b)
        else:
            d2 = tuple(b[q] - a[q] for q in range(3))
            d3 = tuple(c[q] - a[q] for q in range(3))
            self.normal = _normalize(_cross(d2, d3))
            off = _dot(self.normal, tuple(a))
            self.offset = -off if invert else off
        self.invert = 0


class Composite(Obj):
    """composite_object: binary tree of UNION / INTERSECT / DIFFERENCE nodes.

    ``children`` may hold 0, 1 or 2 objects; longer lists are folded into a
    left-deep binary tree.  Difference inverts its right child, as
    composite_object::add_child does.
    """

    def __init__(self, op, children, invert=0, trans=IDENTITY, noop=False):
        assert op in ("union", "intersect", "difference")
        children = list(children)
        if len(children) > 2:
            head = Composite(op, children[:-1])
            children = [head, children[-1]]
        self.op = op
        self.children = children
        self.invert = invert
        self.trans = trans
        self.noop = noop
        if op == "difference" and len(children) == 2:
            children[1].invert = 1

    # ---- flattening
    def program(self):
        """Postfix program (list of sj_csg_node) of this tree."""
        out = []
        _emit(self, IDENTITY, out)
        return out


def Union(*objs, **kw):
    return Composite("union", objs, **kw)


def Intersect(*objs, **kw):
    return Composite("intersect", objs, **kw)


def Difference(a, b, **kw):
    return Composite("difference", [a, b], **kw)


def _node(op, invert=0, m=IDENTITY, t=IDENTITY, c=(0.0, 0.0, 0.0), p=(0.0, 0.0, 0.0, 0.0)):
    n = _abi.CsgNode()
    n.op = op
    n.invert = invert
    for q in range(9):
        n.m[q] = m[q]
        n.t[q] = t[q]
    for q in range(3):
        n.c[q] = c[q]
    for q in range(4):
        n.p[q] = p[q]
    return n


def _emit(obj, acc, out):
    if isinstance(obj, Composite):
        if obj.noop:
            out.append(_node(_abi.CSG_NOOP))
            return
        inner = _matmul(obj.trans, acc) if obj.trans != IDENTITY else acc
        kids = obj.children
        if not kids:
            out.append(_node(_abi.CSG_CONST, obj.invert))
        elif len(kids) == 1:
            _emit(kids[0], inner, out)
            out.append(_node(_abi.CSG_PASS, obj.invert))
        else:
            _emit(kids[0], inner, out)
            _emit(kids[1], inner, out)
            op = _abi.CSG_UNION if obj.op == "union" else _abi.CSG_INTERSECT
            out.append(_node(op, obj.invert))
    elif isinstance(obj, Box):
        out.append(_node(_abi.CSG_BOX, obj.invert, acc, obj.trans, obj.center, obj.offset + (0.0,)))
    elif isinstance(obj, Sphere):
        out.append(_node(_abi.CSG_SPHERE, obj.invert, acc, obj.trans, obj.center, (obj.rad, 0, 0, 0)))
    elif isinstance(obj, Cylinder):
        out.append(_node(_abi.CSG_CYLINDER, obj.invert, acc, obj.trans, obj.center,
                         (obj.height, obj.r1_sq, obj.r2_sq, 0.0)))
    elif isinstance(obj, Plane):
        out.append(_node(_abi.CSG_PLANE, 0, acc, IDENTITY, (0, 0, 0), obj.normal + (obj.offset,)))
    else:
        raise TypeError(f"not a CSG object: {obj!r}")


class Program(Obj):
    """A postfix program given node by node: what a caller that flattens the
    reference's own composite_object trees (the integration walk) passes.
    Nodes are sj_csg_node structures or dicts with the same fields."""

    def __init__(self, nodes):
        self.nodes = [n if isinstance(n, _abi.CsgNode)
                      else _node(n["op"], n["invert"], n["m"], n["t"], n["c"], n["p"]) for n in nodes]

    def program(self):
        return list(self.nodes)


def as_program(obj):
    """Postfix program of any object (a bare primitive becomes a one-node program)."""
    if isinstance(obj, (Composite, Program)):
        return obj.program()
    out = []
    _emit(obj, IDENTITY, out)
    return out
