"""Gmsh mesh files to processed meshes (the reader half of the reference's
preprocessor, tools/pyMeshFV3D: pymeshfv3d/readers/gmsh.py reading, process.py
building faces and geometry).

Reads ASCII MSH 4.1, the format the reference's preprocessor reads
(reader/gmsh.py:35-128: $MeshFormat 4.1 0 8, $PhysicalNames, $Entities, and
the block-structured $Nodes and $Elements, an element's physical group being
the first physical tag of its entity), and the older ASCII MSH 2.2
($PhysicalNames, $Nodes, $Elements with the physical tag on each element);
both give the same processed mesh.  Volume elements become cells: 4-node
tetrahedra (type 4), 8-node hexahedra (5), 6-node prisms (6) and 5-node
pyramids (7), the element kinds of the
preprocessor (utilities/element.py), mixed freely; surface elements (4-node
quadrangles, type 3, or 3-node triangles, type 2) carry the physical group
of the boundary faces they cover.  Regions are numbered as the
reference's processed meshes number them: region 0 the flow domain, then the
boundary physical groups in ascending tag order.

Periodic meshes ($Periodic, translational links) are an extension: the
reference's preprocessor has none.  Every slave node is replaced by its
master (chains of links followed to the end) and the cell keeps the
translation between the two as its vertex shift, so the two cells across a
periodic surface share the face and see each other's centre through the
periodic image (the periodic faces of ``meshgen``).  Surface elements on
periodic surfaces then cover interior faces; physical groups left with no
boundary face get no region.
"""
from __future__ import annotations

import numpy as np

from . import meshgen as mg

_VOLUME = {4: ("tet", 4), 5: ("hex", 8), 6: ("prism", 6), 7: ("pyramid", 5)}
_ETYPE = {kind: t for t, (kind, _) in _VOLUME.items()}
_SURFACE = {3: 4, 2: 3}


def _sections(text):
    out, lines, i = {}, text.splitlines(), 0
    while i < len(lines):
        line = lines[i].strip()
        if line.startswith("$") and not line.startswith("$End"):
            name = line[1:]
            j = i + 1
            while j < len(lines) and lines[j].strip() != f"$End{name}":
                j += 1
            if j == len(lines):
                raise ValueError(f"unterminated section ${name}")
            out[name] = lines[i + 1:j]
            i = j + 1
        else:
            i += 1
    return out


def _periodic_links(lines):
    """(slave id, master id) node pairs of a $Periodic section, with the link
    each pair belongs to."""
    n_links, i, pairs = int(lines[0]), 1, []
    for link in range(n_links):
        i += 1                                   # dimension slave-tag master-tag
        if lines[i].split()[0] == "Affine":      # transformation line (newer writers)
            i += 1
        n = int(lines[i]); i += 1
        for line in lines[i:i + n]:
            sl, ms = line.split()[:2]
            pairs.append((int(sl), int(ms), link))
        i += n
    return pairs


def _resolve_periodic(pairs, index, xyz):
    """Per node row: its canonical row (the end of its chain of links) and the
    translation from that node to this one."""
    master = {}
    for sl, ms, _ in pairs:
        if sl != ms:
            master[index[sl]] = index[ms]
    n = xyz.shape[0]
    root = np.arange(n)
    for v in master:
        r, seen = v, {v}
        while r in master:
            r = master[r]
            if r in seen:
                raise ValueError("cyclic periodic links")
            seen.add(r)
        root[v] = r
    span = np.ptp(xyz, axis=0).max() if n else 1.0
    by_link = {}
    for sl, ms, link in pairs:
        by_link.setdefault(link, []).append(xyz[index[sl]] - xyz[index[ms]])
    for d in by_link.values():
        d = np.asarray(d)
        if np.abs(d - d[0]).max() > 1e-9 * max(span, 1e-300):
            raise ValueError("only translational periodic links are supported")
    return root


def _phys_names(sec):
    out = {}
    for line in sec.get("PhysicalNames", [])[1:]:
        dim, tag, nm = line.split(maxsplit=2)
        out[(int(dim), int(tag))] = nm.strip().strip('"')
    return out


def _parse_22(sec):
    """MSH 2.2: node ids and coordinates, elements as (type, physical tag,
    node ids), periodic (slave, master, link) node pairs."""
    node_lines = sec["Nodes"]
    n_nodes = int(node_lines[0])
    ids = np.empty(n_nodes, dtype=np.int64)
    xyz = np.empty((n_nodes, 3))
    for k, line in enumerate(node_lines[1:1 + n_nodes]):
        p = line.split()
        ids[k] = int(p[0])
        xyz[k] = [float(p[1]), float(p[2]), float(p[3])]
    elements = []
    el_lines = sec["Elements"]
    for line in el_lines[1:1 + int(el_lines[0])]:
        p = [int(v) for v in line.split()]
        etype, ntags = p[1], p[2]
        tags = p[3:3 + ntags]
        elements.append((etype, tags[0] if ntags > 0 else 0, p[3 + ntags:]))
    pairs = _periodic_links(sec["Periodic"]) if "Periodic" in sec else []
    return ids, xyz, elements, pairs


def _parse_41(sec):
    """MSH 4.1 (reader/gmsh.py:57-128 of the reference's preprocessor): the
    physical tag of an element is the first physical tag of its entity (0
    when the entity has none), and elements are ordered by their tags, as
    the reference's reader stores element tag t at position t - 1."""
    phys = {}
    if "Entities" in sec:
        lines = sec["Entities"]
        counts = [int(x) for x in lines[0].split()]
        if len(counts) != 4:
            raise ValueError(f"$Entities: four counts expected, got {lines[0]!r}")
        k = 1
        for dim in range(4):
            for _ in range(counts[dim]):
                t = lines[k].split()
                k += 1
                at = 4 if dim == 0 else 7        # points: tag x y z n tags..., others: a bounding box first
                n_tags = int(t[at])
                phys[(dim, int(t[0]))] = int(t[at + 1]) if n_tags > 0 else 0
    lines = sec["Nodes"]
    n_blocks, n_nodes = [int(x) for x in lines[0].split()[:2]]
    ids = np.empty(n_nodes, dtype=np.int64)
    xyz = np.empty((n_nodes, 3))
    k, row = 1, 0
    for _ in range(n_blocks):
        _, _, parametric, n = [int(x) for x in lines[k].split()]
        if parametric:
            raise ValueError("parametric node coordinates are not supported")
        k += 1
        for i in range(n):
            ids[row + i] = int(lines[k + i])
        for i in range(n):
            p = lines[k + n + i].split()
            xyz[row + i] = [float(p[0]), float(p[1]), float(p[2])]
        k += 2 * n
        row += n
    if row != n_nodes:
        raise ValueError(f"$Nodes: {row} nodes in the blocks, {n_nodes} announced")
    lines = sec["Elements"]
    n_blocks, n_elems = [int(x) for x in lines[0].split()[:2]]
    elements = []
    k = 1
    for _ in range(n_blocks):
        dim, tag, etype, n = [int(x) for x in lines[k].split()]
        k += 1
        ph = phys.get((dim, tag), 0)
        for line in lines[k:k + n]:
            p = [int(v) for v in line.split()]
            elements.append((p[0], etype, ph, p[1:]))
        k += n
    if len(elements) != n_elems:
        raise ValueError(f"$Elements: {len(elements)} elements in the blocks, {n_elems} announced")
    elements.sort(key=lambda e: e[0])
    elements = [e[1:] for e in elements]
    pairs = []
    if "Periodic" in sec:
        lines = sec["Periodic"]
        k = 1
        for link in range(int(lines[0])):
            k += 1                               # entity dimension, tag, master tag
            k += 1                               # the affine transformation: count and values
            n = int(lines[k])
            k += 1
            for line in lines[k:k + n]:
                sl, ms = line.split()[:2]
                pairs.append((int(sl), int(ms), link))
            k += n
    return ids, xyz, elements, pairs


def read_msh(path_or_text, name=None, scale=(1.0, 1.0, 1.0)):
    """A processed ``meshgen.Mesh`` from an ASCII MSH 4.1 or 2.2 file (or
    its text)."""
    text = path_or_text
    if "\n" not in path_or_text:
        with open(path_or_text) as f:
            text = f.read()
    sec = _sections(text)
    fmt = sec.get("MeshFormat", ["?"])[0].split()
    version = fmt[0] if fmt else "?"
    if len(fmt) > 1 and fmt[1] != "0":
        raise ValueError("binary MSH files are not supported")
    if version == "4.1":
        ids, xyz, elements, pairs = _parse_41(sec)
    elif version.startswith("2"):
        ids, xyz, elements, pairs = _parse_22(sec)
    else:
        raise ValueError(f"MSH format {version} not supported (ASCII 4.1 or 2.2)")
    phys_names = _phys_names(sec)
    xyz *= np.asarray(scale, dtype=float)
    index = {int(t): k for k, t in enumerate(ids)}
    cells, kinds, surf = [], [], []
    for etype, phys, nodes in elements:
        conn = [index[v] for v in nodes]
        if etype in _VOLUME:
            kind, nv = _VOLUME[etype]
            kinds.append(kind)
            cells.append(conn[:nv] + [-1] * (8 - nv))
        elif etype in _SURFACE:
            surf.append((phys, conn[:_SURFACE[etype]]))
        elif etype in (1, 15):          # lines, points: geometry only
            continue
        else:
            raise ValueError(f"Gmsh element type {etype} not supported")
    if not cells:
        raise ValueError("no volume elements")
    cell_nodes = np.asarray(cells, dtype=np.int64)
    width = max(_VOLUME[_ETYPE[k]][1] for k in set(kinds))
    cell_nodes = cell_nodes[:, :width]
    valid = cell_nodes >= 0
    shift = np.zeros(cell_nodes.shape + (3,))
    if pairs:
        root = _resolve_periodic(pairs, index, xyz)
        canon = np.where(valid, root[np.maximum(cell_nodes, 0)], -1)
        shift[valid] = xyz[cell_nodes[valid]] - xyz[canon[valid]]
        cell_nodes = canon
        surf = [(t, [int(root[v]) for v in c]) for t, c in surf]
        # surfaces that cover faces between two cells now are not boundaries
        count = {}
        for c, kind in zip(cell_nodes, kinds):
            for face in mg.KINDS[kind][1]:
                key = tuple(sorted(int(v) for v in c[face]))
                count[key] = count.get(key, 0) + 1
        surf = [(t, c) for t, c in surf if count.get(tuple(sorted(c)), 0) == 1]
    tags = sorted({t for t, _ in surf})
    region_of_tag = {t: r + 1 for r, t in enumerate(tags)}
    names = ["flow"] + [phys_names.get((2, t), f"boundary{t}") for t in tags]
    # boundary faces are matched to surface elements by their node sets
    surf_key = {tuple(sorted(c)): region_of_tag[t] for t, c in surf}

    def regions(face_nodes):
        out = np.empty(face_nodes.shape[0], dtype=np.int64)
        for i, row in enumerate(face_nodes):
            key = tuple(int(v) for v in row if v >= 0)   # triangles of mixed meshes: leading -1
            r = surf_key.get(key)
            if r is None:
                raise ValueError(f"boundary face with nodes {[int(ids[v]) for v in key]} has no physical surface")
            out[i] = r
        return out

    kind = kinds[0] if len(set(kinds)) == 1 else kinds
    return mg.build_mesh(xyz, cell_nodes, shift, kind,
                         boundary_region_of_nodes=regions if surf else None,
                         region_names=tuple(names), region_is_boundary=tuple([0] + [1] * len(tags)),
                         name=name or "gmsh")


def write_msh(path, nodes, cell_nodes, cell_kind, boundary, phys_names, periodic=None, version="4.1"):
    """Write an ASCII MSH file (version "4.1" or "2.2"): nodes (n, 3), volume
    connectivity (rows padded with -1 for mixed kinds; cell_kind one kind or
    one per cell), the boundary surface elements as (physical tag, node
    list) pairs, and optionally periodic links, each a list of (slave node,
    master node) pairs (0-based) related by one translation."""
    kinds = [cell_kind] * len(cell_nodes) if isinstance(cell_kind, str) else list(cell_kind)
    vol_tag = max([t for (d, t) in phys_names if d == 3], default=0)
    if version == "2.2":
        lines = _write_22(nodes, cell_nodes, kinds, boundary, phys_names, periodic, vol_tag)
    elif version == "4.1":
        lines = _write_41(nodes, cell_nodes, kinds, boundary, phys_names, periodic, vol_tag)
    else:
        raise ValueError(f"MSH version {version} cannot be written (4.1 or 2.2)")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def _names(phys_names, fmt):
    lines = ["$MeshFormat", fmt, "$EndMeshFormat", "$PhysicalNames", str(len(phys_names))]
    for (dim, tag), nm in sorted(phys_names.items()):
        lines.append(f'{dim} {tag} "{nm}"')
    return lines + ["$EndPhysicalNames"]


def _write_22(nodes, cell_nodes, kinds, boundary, phys_names, periodic, vol_tag):
    lines = _names(phys_names, "2.2 0 8") + ["$Nodes", str(nodes.shape[0])]
    for k, x in enumerate(nodes):
        lines.append(f"{k + 1} {float(x[0])!r} {float(x[1])!r} {float(x[2])!r}")
    lines += ["$EndNodes", "$Elements", str(len(boundary) + cell_nodes.shape[0])]
    eid = 1
    for tag, conn in boundary:
        st = 3 if len(conn) == 4 else 2
        lines.append(" ".join(str(int(v)) for v in [eid, st, 2, tag, tag] + [int(c) + 1 for c in conn]))
        eid += 1
    for conn, kind in zip(cell_nodes, kinds):
        etype = _ETYPE[kind]
        nv = _VOLUME[etype][1]
        lines.append(" ".join(str(v) for v in [eid, etype, 2, vol_tag, vol_tag] + [int(c) + 1 for c in conn[:nv]]))
        eid += 1
    lines.append("$EndElements")
    if periodic:
        lines += ["$Periodic", str(len(periodic))]
        for k, link in enumerate(periodic):
            lines += [f"2 {2 * k + 1} {2 * k + 2}", str(len(link))]
            lines += [f"{int(a) + 1} {int(b) + 1}" for a, b in link]
        lines.append("$EndPeriodic")
    return lines


def _write_41(nodes, cell_nodes, kinds, boundary, phys_names, periodic, vol_tag):
    """MSH 4.1: one surface entity per boundary physical tag (entity tag =
    physical tag), two untagged surface entities per periodic link, one
    volume entity (tag 1) holding every node and cell."""
    lo, hi = nodes.min(axis=0), nodes.max(axis=0)
    box = " ".join(repr(float(v)) for v in (*lo, *hi))
    surf_tags = sorted({int(t) for t, _ in boundary})
    links = periodic or []
    per_tags = [(100000 + 2 * k + 1, 100000 + 2 * k + 2) for k in range(len(links))]
    lines = _names(phys_names, "4.1 0 8")
    lines += ["$Entities", f"0 0 {len(surf_tags) + 2 * len(links)} 1"]
    lines += [f"{t} {box} 1 {t} 0" for t in surf_tags]
    lines += [f"{t} {box} 0 0" for pair in per_tags for t in pair]
    lines += [f"1 {box} " + (f"1 {vol_tag} 0" if vol_tag else "0 0"), "$EndEntities"]
    n = nodes.shape[0]
    lines += ["$Nodes", f"1 {n} 1 {n}", f"3 1 0 {n}"]
    lines += [str(k + 1) for k in range(n)]
    lines += [f"{float(x[0])!r} {float(x[1])!r} {float(x[2])!r}" for x in nodes]
    lines.append("$EndNodes")
    # element tags: the boundary elements 1.. in the order given, then the
    # cells in their order (which the processed mesh keeps); blocks group
    # them by entity and type
    nbd = len(boundary)
    blocks = []
    for t in surf_tags:
        for st, nv in ((2, 3), (3, 4)):
            rows = [(e + 1, c) for e, (tag, c) in enumerate(boundary) if int(tag) == t and len(c) == nv]
            if rows:
                blocks.append((2, t, st, rows))
    for kind in sorted(set(kinds), key=lambda k_: _ETYPE[k_]):
        etype = _ETYPE[kind]
        nv = _VOLUME[etype][1]
        rows = [(nbd + i + 1, conn[:nv]) for i, (conn, k_) in enumerate(zip(cell_nodes, kinds)) if k_ == kind]
        blocks.append((3, 1, etype, rows))
    total = sum(len(b[3]) for b in blocks)
    lines += ["$Elements", f"{len(blocks)} {total} 1 {total}"]
    for dim, tag, etype, rows in blocks:
        lines.append(f"{dim} {tag} {etype} {len(rows)}")
        for eid, conn in rows:
            lines.append(" ".join(str(int(v)) for v in [eid] + [int(c) + 1 for c in conn]))
    lines.append("$EndElements")
    if links:
        lines += ["$Periodic", str(len(links))]
        for (slave, master), link in zip(per_tags, links):
            a, b = link[0]
            t = nodes[a] - nodes[b]
            affine = [1, 0, 0, t[0], 0, 1, 0, t[1], 0, 0, 1, t[2], 0, 0, 0, 1]
            lines += [f"2 {slave} {master}", "16 " + " ".join(repr(float(v)) for v in affine), str(len(link))]
            lines += [f"{int(a) + 1} {int(b) + 1}" for a, b in link]
        lines.append("$EndPeriodic")
    return lines
