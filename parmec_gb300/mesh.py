"""MESH (input.cpp:840-1156) with MESH_Create / MESH_Char (mesh.cpp:255-521).

A MESH is one rigid particle built from volume elements (tetrahedra,
pyramids, wedges, hexahedra).  Its boundary faces become nodes, faces and
triangles of the particle (triangles carry triobs = the particle, so spheres
touch them as a particle), and its mass, centroid and inertia come from
integrating the density over the elements.

The order of faces, and so of triangles, is the reference's: elements are
taken in input order; a face seen a second time is an inner face; the
boundary faces of each surface element keep the order in which they were
created; and the mesh face list holds them last element first (the reference
prepends to singly linked lists, mesh.cpp:208-241, 372-446).
"""
import numpy as np

# local faces of each element type, as 1-based positions in the element's node
# list, oriented outwards; a trailing 0 pads triangles (mesh.cpp:40-61)
_FACES = {
    4: ((1, 3, 2, 0), (1, 2, 4, 0), (2, 3, 4, 0), (3, 1, 4, 0)),
    5: ((1, 4, 3, 2), (1, 2, 5, 0), (2, 3, 5, 0), (3, 4, 5, 0), (4, 1, 5, 0)),
    6: ((1, 3, 2, 0), (4, 5, 6, 0), (1, 2, 5, 4), (2, 3, 6, 5), (3, 1, 4, 6)),
    8: ((1, 4, 3, 2), (1, 2, 6, 5), (2, 3, 7, 6), (3, 4, 8, 7), (1, 5, 8, 4), (5, 6, 7, 8)),
}


def _face_size(etype, n):
    """Nodes of local face n (setup_face, mesh.cpp:134-182)."""
    if etype == 4:
        return 3
    if etype == 5:
        return 4 if n == 0 else 3
    if etype == 6:
        return 3 if n < 2 else 4
    return 4


def _face_nodes(ele, n):
    k = _face_size(ele["type"], n)
    return [ele["nodes"][_FACES[ele["type"]][n][m] - 1] for m in range(k)]


def parse(nodes, elements, colors):
    """Argument checks and parsing of MESH (input.cpp:840-995)."""
    if not isinstance(nodes, list) or not isinstance(elements, list):
        raise TypeError("'nodes' and 'elements' must be lists")
    if not (isinstance(colors, list) or isinstance(colors, (int, float))):
        raise TypeError("'colors' must be a list or a number")
    i, n = 0, len(elements)
    while i < n:
        k = int(elements[i])
        if k not in (4, 5, 6, 8):
            raise ValueError("An element must have 4, 5, 6, or 8 nodes")
        i += k + 1
        if i >= n:
            raise ValueError("The last element definition is incomplete")
        i += 1
    if len(nodes) % 3:
        raise ValueError("Nodes list length must be a multiple of 3")
    nn = len(nodes) // 3
    eles = []
    i = 0
    while i < n:
        k = int(elements[i])
        ids = [int(v) for v in elements[i + 1:i + 1 + k]]
        for j, v in enumerate(ids):
            if v < 0 or v >= nn:
                raise ValueError(f"Node {j} in element {len(eles)} is outside of range [0, {nn - 1}]")
        if len(set(ids)) != k:
            raise ValueError(f"Nodes in element {len(eles)} repeat")
        eles.append((ids, int(elements[i + 1 + k])))
        i += k + 2
    if isinstance(colors, list):
        gcolor = int(colors[0])
        faces = []
        i, n = 1, len(colors)
        while i < n:
            k = int(colors[i])
            if k not in (3, 4):
                raise ValueError("A face must have 3 or 4 nodes")
            if i + k + 1 >= n:
                raise ValueError("The last face definition is incomplete")
            ids = [int(v) for v in colors[i + 1:i + 1 + k]]
            for j, v in enumerate(ids):
                if v < 0 or v >= nn:
                    raise ValueError(f"Node {j} in face {len(faces)} is outside of range [0, {nn - 1}]")
            if len(set(ids)) != k:
                raise ValueError(f"Nodes in face {len(faces)} repeat")
            faces.append((ids, int(colors[i + 1 + k])))
            i += k + 2
    else:
        gcolor, faces = int(colors), []
    xyz = [[float(nodes[3 * j + c]) for c in range(3)] for j in range(nn)]
    return xyz, eles, gcolor, faces


def create(xyz, eles, gcolor, surf):
    """MESH_Create (mesh.cpp:310-470): nodes, surface/bulk elements and the
    boundary face list (nodes local to the mesh, 0-based from the smallest)."""
    fmap = {}
    flist = []                                   # creation order
    elist = []
    for ids, mat in eles:
        ele = {"type": len(ids), "nodes": list(ids), "mat": mat, "neighs": 0, "faces": []}
        for n in range(len(_FACES[ele["type"]])):
            f = _face_nodes(ele, n)
            key = (len(f), tuple(sorted(f)))
            hit = fmap.get(key)
            if hit is not None:
                ele["neighs"] += 1
                if hit["ele"] is not None:
                    hit["ele"]["neighs"] += 1
                hit["ele"] = None                # an inner face
            else:
                rec = {"ele": ele, "index": n, "key": key}
                fmap[key] = rec
                flist.append(rec)
        elist.append(ele)
    lo = min(min(ids) for ids, _ in eles)
    hi = max(max(ids) for ids, _ in eles)
    for ele in elist:
        ele["nodes"] = [v - lo for v in ele["nodes"]]
    surfeles = [e for e in elist if e["neighs"] < len(_FACES[e["type"]])]
    bulkeles = [e for e in elist if e["neighs"] >= len(_FACES[e["type"]])]
    smap = {}
    for ids, color in surf:
        smap[(len(ids), tuple(sorted(ids)))] = color
    # boundary faces: each element's list ends up in creation order
    for rec in reversed(flist):
        ele = rec["ele"]
        if ele is None:
            continue
        ele["faces"].insert(0, {"nodes": _face_nodes(ele, rec["index"]), "color": smap.get(rec["key"], gcolor)})
    faces = []
    for ele in surfeles:
        for f in ele["faces"]:
            faces.insert(0, f)
    nodes = [list(xyz[j]) for j in range(lo, hi + 1)]
    return {"nodes": nodes, "faces": faces, "surfeles": surfeles, "bulkeles": bulkeles}


def _simplex(a, b, c, d):
    """Volume, first and second moments of the tetrahedron (a, b, c, d) scaled
    by J = det[b-a, c-a, d-a] (simplex.h:33-116, evaluated in the same order)."""
    q = [b[0] - a[0], c[0] - a[0], d[0] - a[0], b[1] - a[1], c[1] - a[1], d[1] - a[1],
         b[2] - a[2], c[2] - a[2], d[2] - a[2]]
    J = (q[0] * q[4] * q[8] + q[3] * q[7] * q[2] + q[6] * q[1] * q[5]
         - q[6] * q[4] * q[2] - q[0] * q[7] * q[5] - q[3] * q[1] * q[8])
    return J


def _second(J, a, b, c, d, i, k):
    p = (a, b, c, d)
    s = None
    for m in range(4):
        for n in range(4):
            t = (2. * p[m][i] * p[n][k]) if m == n else (p[m][i] * p[n][k])
            s = t if s is None else s + t
    return (J / 120.) * s


def characterize(msh, density):
    """MESH_Char (mesh.cpp:486-518) with element_char_add (255-308): mass,
    mass centre and inertia tensor (column-major 3x3)."""
    me = sx = sy = sz = 0.0
    euler = [0.0] * 9
    zero = msh["nodes"][0]
    for ele in msh["bulkeles"] + msh["surfeles"]:
        rho = density(ele["mat"])
        et = ele["type"]
        for i in range(len(_FACES[et])):
            # vertices of face i; the reference counts 4 for every tetrahedron
            # face and so reads one node past the table there, 3 are used here
            nv = _face_size(et, i)
            ver = _FACES[et][i]
            a = msh["nodes"][ele["nodes"][ver[0] - 1]]
            for j in range(1, nv - 1):
                b = msh["nodes"][ele["nodes"][ver[j] - 1]]
                c = msh["nodes"][ele["nodes"][ver[j + 1] - 1]]
                J = rho * _simplex(zero, a, b, c)
                me += J / 6.
                sx += (J / 24.) * (zero[0] + a[0] + b[0] + c[0])
                sy += (J / 24.) * (zero[1] + a[1] + b[1] + c[1])
                sz += (J / 24.) * (zero[2] + a[2] + b[2] + c[2])
                euler[0] += _second(J, zero, a, b, c, 0, 0)
                euler[3] += _second(J, zero, a, b, c, 0, 1)
                euler[4] += _second(J, zero, a, b, c, 1, 1)
                euler[6] += _second(J, zero, a, b, c, 0, 2)
                euler[7] += _second(J, zero, a, b, c, 1, 2)
                euler[8] += _second(J, zero, a, b, c, 2, 2)
    center = [sx / me, sy / me, sz / me]
    euler[0] -= (2 * sx - center[0] * me) * center[0]
    euler[4] -= (2 * sy - center[1] * me) * center[1]
    euler[8] -= (2 * sz - center[2] * me) * center[2]
    euler[3] -= center[0] * sy + center[1] * sx - center[0] * center[1] * me
    euler[6] -= center[0] * sz + center[2] * sx - center[0] * center[2] * me
    euler[7] -= center[1] * sz + center[2] * sy - center[1] * center[2] * me
    euler[1] = euler[3]
    euler[2] = euler[6]
    euler[5] = euler[7]
    trace = euler[0] + euler[4] + euler[8]
    ident = [1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0]
    inertia = [ident[k] * trace - euler[k] for k in range(9)]
    return me, center, inertia


def mesh_command(m, nodes, elements, material, colors):
    """Append one MESH particle to model m; returns its particle index."""
    from .model import OUTREST, _invert
    if not (0 <= int(material) < len(m.mparam)):
        raise ValueError("'material' out of range")
    xyz, eles, gcolor, surf = parse(nodes, elements, colors)
    for _, mat in eles:
        if not (0 <= mat < len(m.mparam)):
            raise ValueError("element material out of range")
    msh = create(xyz, eles, gcolor, surf)
    ip = m.parnum                               # the particle these nodes and faces belong to
    # faces and triangles (input.cpp:1034-1085)
    N, F, T = m.N, m.F, m.Tr
    nod0 = m.nodnum
    for fac in msh["faces"]:
        quads = [(0, 1, 2)] + ([(0, 2, 3)] if len(fac["nodes"]) == 4 else [])
        for q in quads:
            t = m.trinum
            T.ensure(t + 1)
            m.trinum += 1
            for v in range(3):
                T.tri[3 * v:3 * v + 3, t] = msh["nodes"][fac["nodes"][q[v]]]
            T.tricol[t] = fac["color"]
            T.triobs[t] = ip
            f = m.facnum
            F.ensure(f + 1)
            m.facnum += 1
            for v in range(3):
                F.facnod[v, f] = nod0 + fac["nodes"][q[v]]
            F.factri[f] = t
    # nodes (input.cpp:1087-1095)
    for j, xyz_j in enumerate(msh["nodes"]):
        k = m.nodnum
        N.ensure(k + 1)
        m.nodnum += 1
        N.nodes[0:3, k] = xyz_j
        N.nodes[3:6, k] = xyz_j
        N.nodpart[k] = ip
    # the particle (input.cpp:1097-1150)
    i = m._new_particle()
    P = m.P
    P.parmat[i] = int(material)
    mass, center, inertia = characterize(msh, lambda k: m.mparam[k][0])
    P.position[0:3, i] = center
    P.position[3:6, i] = center
    P.mass[i] = mass
    P.invm[i] = 1.0 / mass
    P.rotation[:, i] = [1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0]
    P.inertia[:, i] = inertia
    P.inverse[:, i] = _invert(inertia)
    P.flags[i] = OUTREST
    return i


def hexahedron(x0, y0, z0, a):
    """Nodes and the element list of one a x a x a hexahedron at (x0, y0, z0)
    (node order of the reference's hexahedron: bottom face 0-3, top face 4-7)."""
    c = [(x0, y0, z0), (x0 + a, y0, z0), (x0 + a, y0 + a, z0), (x0, y0 + a, z0),
         (x0, y0, z0 + a), (x0 + a, y0, z0 + a), (x0 + a, y0 + a, z0 + a), (x0, y0 + a, z0 + a)]
    nodes = [v for p in c for v in p]
    return nodes, [8, 0, 1, 2, 3, 4, 5, 6, 7, 0]


def hex_grid(m, origins, a, material, color):
    """MESH of one a-sided hexahedron at every origin (an (n, 3) array), the
    same as n separate MESH commands: the face topology is built once and the
    mass integrals are evaluated for all cubes at once in the same operation
    order (numpy float64 arithmetic, element by element).  Returns the
    particle indices."""
    from .model import OUTREST, _invert
    origins = np.asarray(origins, dtype=np.float64)
    n = len(origins)
    nodes0, ele0 = hexahedron(0.0, 0.0, 0.0, a)
    xyz, eles, gcolor, surf = parse(nodes0, ele0[:-1] + [material], color)
    msh = create(xyz, eles, gcolor, surf)
    # node coordinates of every cube, (n, 8, 3), built as hexahedron() builds them
    ox, oy, oz = origins[:, 0], origins[:, 1], origins[:, 2]
    X = np.stack([ox, ox + a, ox + a, ox, ox, ox + a, ox + a, ox], axis=1)
    Y = np.stack([oy, oy, oy + a, oy + a, oy, oy, oy + a, oy + a], axis=1)
    Z = np.stack([oz, oz, oz, oz, oz + a, oz + a, oz + a, oz + a], axis=1)
    C = np.stack([X, Y, Z], axis=2)
    # triangles and faces, in the order of one MESH command, cube after cube
    tris = []
    for fac in msh["faces"]:
        tris.append((fac["nodes"][0], fac["nodes"][1], fac["nodes"][2], fac["color"]))
        if len(fac["nodes"]) == 4:
            tris.append((fac["nodes"][0], fac["nodes"][2], fac["nodes"][3], fac["color"]))
    nt, nn = len(tris), 8
    t0, f0, n0, p0 = m.trinum, m.facnum, m.nodnum, m.parnum
    m.Tr.ensure(t0 + n * nt)
    m.F.ensure(f0 + n * nt)
    m.N.ensure(n0 + n * nn)
    m.P.ensure(p0 + n)
    parts = p0 + np.arange(n)
    for q, (u, v, w, col) in enumerate(tris):
        t = t0 + np.arange(n) * nt + q
        for vi, node in enumerate((u, v, w)):
            m.Tr.tri[3 * vi:3 * vi + 3, t] = C[:, node, :].T
            m.F.facnod[vi, f0 + np.arange(n) * nt + q] = n0 + np.arange(n) * nn + node
        m.Tr.tricol[t] = col
        m.Tr.triobs[t] = parts
        m.F.factri[f0 + np.arange(n) * nt + q] = t
    for j in range(nn):
        k = n0 + np.arange(n) * nn + j
        m.N.nodes[0:3, k] = C[:, j, :].T
        m.N.nodes[3:6, k] = C[:, j, :].T
        m.N.nodpart[k] = parts
    m.trinum += n * nt
    m.facnum += n * nt
    m.nodnum += n * nn
    # mass properties (characterize() on arrays)
    rho = m.mparam[material][0]
    me = sx = sy = sz = np.zeros(n)
    eu = [np.zeros(n) for _ in range(9)]
    zero = C[:, 0, :]
    ele = msh["surfeles"][0]
    for i in range(len(_FACES[8])):
        ver = _FACES[8][i]
        A = C[:, ele["nodes"][ver[0] - 1], :]
        for j in range(1, _face_size(8, i) - 1):
            B = C[:, ele["nodes"][ver[j] - 1], :]
            D = C[:, ele["nodes"][ver[j + 1] - 1], :]
            J = rho * _simplex(zero.T, A.T, B.T, D.T)
            me = me + J / 6.
            sx = sx + (J / 24.) * (zero[:, 0] + A[:, 0] + B[:, 0] + D[:, 0])
            sy = sy + (J / 24.) * (zero[:, 1] + A[:, 1] + B[:, 1] + D[:, 1])
            sz = sz + (J / 24.) * (zero[:, 2] + A[:, 2] + B[:, 2] + D[:, 2])
            for k, (ii, kk) in ((0, (0, 0)), (3, (0, 1)), (4, (1, 1)), (6, (0, 2)), (7, (1, 2)), (8, (2, 2))):
                eu[k] = eu[k] + _second(J, zero.T, A.T, B.T, D.T, ii, kk)
    center = [sx / me, sy / me, sz / me]
    eu[0] = eu[0] - (2 * sx - center[0] * me) * center[0]
    eu[4] = eu[4] - (2 * sy - center[1] * me) * center[1]
    eu[8] = eu[8] - (2 * sz - center[2] * me) * center[2]
    eu[3] = eu[3] - (center[0] * sy + center[1] * sx - center[0] * center[1] * me)
    eu[6] = eu[6] - (center[0] * sz + center[2] * sx - center[0] * center[2] * me)
    eu[7] = eu[7] - (center[1] * sz + center[2] * sy - center[1] * center[2] * me)
    eu[1], eu[2], eu[5] = eu[3], eu[6], eu[7]
    trace = eu[0] + eu[4] + eu[8]
    ident = [1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0]
    P = m.P
    m.parnum += n
    P.angular[:, parts] = 0.0
    P.linear[:, parts] = 0.0
    P.force[:, parts] = 0.0
    P.torque[:, parts] = 0.0
    P.parmat[parts] = material
    for c in range(3):
        P.position[c, parts] = center[c]
        P.position[3 + c, parts] = center[c]
    P.mass[parts] = me
    P.invm[parts] = 1.0 / me
    P.rotation[:, parts] = np.array(ident)[:, None]
    inertia = np.stack([ident[k] * trace - eu[k] for k in range(9)])
    P.inertia[:, parts] = inertia
    for q, p in enumerate(parts):
        P.inverse[:, p] = _invert(inertia[:, q])
    P.flags[parts] = OUTREST
    m._touch()
    return parts


def mesh_contact_grid(m):
    """Grid cell and big-triangle flags of the mesh-mesh contact search
    (pg_session_mesh_contact): a triangle's box, widened by the swept radius
    r on each side, spans at most its longest edge + 2r along any axis
    whatever its rotation; triangles up to 4 times the median of that bound
    set the cell (the largest of them), longer ones are "big" and searched
    against every triangle.  Returns (cell, big) with big a uint8 array over
    all triangles (0 for obstacle triangles)."""
    T = m.trinum
    big = np.zeros(max(T, 1), dtype=np.uint8)
    r = float(m.tt_radius)
    own = m.Tr.triobs[:T] >= 0
    if not np.any(own):
        return 2.0 * r if r > 0.0 else 1.0, big
    v = m.Tr.tri[:, :T].reshape(3, 3, T)
    e = [np.sqrt(np.sum((v[a] - v[(a + 1) % 3]) ** 2, axis=0)) for a in range(3)]
    ext = np.maximum(np.maximum(e[0], e[1]), e[2]) + 2.0 * r
    med = float(np.median(ext[own]))
    small = own & (ext <= 4.0 * med)
    cell = float(np.max(ext[small]))
    big[:T] = (own & ~small).astype(np.uint8)
    return cell, big
