"""Spin operators and coupling-position generators (drop-in for T-Nalg's HamiltonianModule).

Same names, return types and numbering as HamiltonianModule.py:8-261 and
library/HamiltonianModule.py:333-349 (husimi); host-side only.
"""
import numpy as np


def spin_operators(spin):
    """[id, sx, sy, sz, su, sd] as a dict (HamiltonianModule.py:8-44). sy is complex."""
    op = dict()
    if spin == "half":
        op["id"] = np.eye(2)
        op["sx"] = np.array([[0.0, 0.5], [0.5, 0.0]])
        op["sy"] = np.array([[0.0, 0.5j], [-0.5j, 0.0]], dtype=complex)
        op["sz"] = np.array([[0.5, 0.0], [0.0, -0.5]])
        op["su"] = np.array([[0.0, 1.0], [0.0, 0.0]])
        op["sd"] = np.array([[0.0, 0.0], [1.0, 0.0]])
    elif spin == "one":
        r = 2 ** -0.5
        op["id"] = np.eye(3)
        op["sx"] = np.array([[0, 1, 0], [1, 0, 1], [0, 1, 0]], dtype=float) * r
        op["sy"] = np.array([[0, -1j, 0], [1j, 0, -1j], [0, 1j, 0]], dtype=complex) * r
        op["sz"] = np.diag([1.0, 0.0, -1.0])
        op["su"] = np.real(op["sx"] + 1j * op["sy"])
        op["sd"] = np.real(op["sx"] - 1j * op["sy"])
    else:
        raise ValueError("spin must be 'half' or 'one'")
    return op


def positions_nearest_neighbor_1d(l, bound_cond="open"):
    """Rows [n, n+1] (+ [0, l-1] if periodic) as floats (HamiltonianModule.py:151-162)."""
    nh = l - 1
    index = np.zeros((nh + (bound_cond == "periodic"), 2))
    index[:nh, 0] = np.arange(nh)
    index[:nh, 1] = np.arange(1, nh + 1)
    if bound_cond == "periodic":
        index[nh] = [0, l - 1]
    return index


def positions_jigsaw_1d(length, bound_cond="open"):
    """Chain bonds plus next-nearest bonds on even sites (HamiltonianModule.py:165-200)."""
    if bound_cond == "open":
        if length % 2 == 0:
            length += 1
        n_half = round((length - 1) / 2)
    else:
        if length % 2 == 1:
            length += 1
        n_half = round(length / 2)
    pos = np.zeros((n_half * 3, 2))
    for n in range(length - 1):
        pos[n] = [n, n + 1]
    l_now = length - 1
    if bound_cond == "periodic":
        pos[l_now] = [0, length - 1]
        l_now += 1
        for n in range(n_half - 1):
            pos[l_now + n] = [2 * n, 2 * (n + 1)]
        pos[n_half * 3 - 1] = [0, length - 2]
    else:
        for n in range(n_half):
            pos[l_now + n] = [2 * n, 2 * (n + 1)]
    return pos


def positions_nearest_neighbor_square(width, height, bound_cond="open"):
    """Row bonds, then column bonds, then periodic wraps (HamiltonianModule.py:203-227)."""
    rows = [[n * width + i, n * width + i + 1] for n in range(height) for i in range(width - 1)]
    cols = [[i * width + n, (i + 1) * width + n] for n in range(width) for i in range(height - 1)]
    pos = np.array(rows + cols, dtype=float).reshape(-1, 2)
    if bound_cond == "periodic":
        wrap = [[n * width, (n + 1) * width - 1] for n in range(height)]
        wrap += [[n, (height - 1) * width + n] for n in range(width)]
        pos = np.vstack((pos, np.array(wrap, dtype=float))).astype(int)
    return pos


def positions_fully_connected(n_site):
    """All pairs n0 < n1 (HamiltonianModule.py:230-239)."""
    return np.array([[a, b] for a in range(n_site - 1) for b in range(a + 1, n_site)], dtype=int).reshape(-1, 2)


def positions_husimi(depth):
    """Husimi-cactus bonds (library/HamiltonianModule.py:333-349).

    A central triangle (0, B+1, 2B+2) with B = sum_{n<depth} 2^(n+1) sites per branch;
    inside branch b every internal site n spawns the triangle (n, 2n+1, 2n+2), all
    offset by b*(B+1). Each triangle contributes bonds [n1,n2], [n2,n3], [n1,n3].
    """
    nb = sum(2 ** (n + 1) for n in range(depth))

    def tri(a, b, c):
        return [[a, b], [b, c], [a, c]]

    pos = tri(0, nb + 1, 2 * nb + 2)
    inner = nb - 2 ** depth
    for br in range(3):
        off = (nb + 1) * br
        for n in range(1, inner + 1):
            pos += tri(n + off, 2 * n + 1 + off, 2 * n + 2 + off)
    return np.array(pos)


def snake_site(x, y, width):
    """Chain index of square-lattice site (x, y) in snake order: even rows left to right, odd rows
    right to left, so that consecutive chain sites are lattice neighbours."""
    return y * width + (x if y % 2 == 0 else width - 1 - x)


def positions_j1j2_square_snake(width, height):
    """Bonds of the J1-J2 model on an open width x height square lattice in snake order.

    Returns (pos_j1, pos_j2): nearest-neighbour bonds (2 w h - w - h of them) and diagonal
    next-nearest-neighbour bonds (2 (w - 1)(h - 1)), each row [i, j] with i < j, rows sorted.
    Not in the reference, which builds such lattices through its 'arbitrary' index lists
    (Parameters.py:205-212); a 6 x 6 lattice gives 60 J1 and 50 J2 bonds, bonds up to 11 sites
    apart along the chain.
    """
    def bond(a, b):
        i, j = snake_site(*a, width), snake_site(*b, width)
        return [min(i, j), max(i, j)]

    j1, j2 = [], []
    for y in range(height):
        for x in range(width):
            if x + 1 < width:
                j1.append(bond((x, y), (x + 1, y)))
            if y + 1 < height:
                j1.append(bond((x, y), (x, y + 1)))
            if x + 1 < width and y + 1 < height:
                j2.append(bond((x, y), (x + 1, y + 1)))
                j2.append(bond((x + 1, y), (x, y + 1)))
    return np.array(sorted(j1), dtype=int).reshape(-1, 2), np.array(sorted(j2), dtype=int).reshape(-1, 2)


def interactions_position2full_index_heisenberg_two_body(index_pos):
    """Each bond -> rows [i, j, su, sd], [i, j, sd, su], [i, j, sz, sz] (HamiltonianModule.py:242-261)."""
    index_pos = np.asarray(index_pos)
    nh = index_pos.shape[0]
    index = np.zeros((nh * 3, 4), dtype=int)
    for n in range(nh):
        i, j = int(index_pos[n, 0]), int(index_pos[n, 1])
        index[3 * n] = [i, j, 4, 5]
        index[3 * n + 1] = [i, j, 5, 4]
        index[3 * n + 2] = [i, j, 3, 3]
    return index
