"""Pure-Python, loop-for-loop restatement of the reference's dictionary <-> vector
coefficient layout, for small cases only.

TEST INFRASTRUCTURE ONLY.  Follows src/dg_vmethods.jl:35-142 (get_size, D2V,
V2D, D2Vref, V2Dref) and src/schemes.jl:21-27 (cutoff), including Julia's
column-major CartesianIndices order (dimension 1 fastest) and 1-based levels.
Dictionaries are keyed by 1-based level tuples; each value is a dict keyed by
cell tuples whose values are dicts keyed by mode tuples.
"""
import itertools


def cartesian(shape):
    """Julia CartesianIndices(shape) order: first index varies fastest, 1-based."""
    for rev in itertools.product(*[range(1, s + 1) for s in reversed(shape)]):
        yield tuple(reversed(rev))


def cutoff(scheme, level, n):
    if scheme == "sparse":
        return sum(level) > n + len(level)
    return False


def get_size(D, k, n, scheme="sparse"):
    size = 0
    for level in cartesian((n + 1,) * D):
        if cutoff(scheme, level, n):
            continue
        ks = 1
        for q in range(D):
            ks *= 1 << max(0, level[q] - 2)
        size += ks * k ** D
    return size


def V2Dref(D, k, n, scheme="sparse"):
    out = []
    for level in cartesian((n + 1,) * D):
        if cutoff(scheme, level, n):
            continue
        ks = tuple(1 << max(0, level[q] - 2) for q in range(D))
        for cell in cartesian(ks):
            for mode in cartesian((k,) * D):
                out.append((level, cell, mode))
    return out


def D2Vref(D, k, n, scheme="sparse"):
    return {lcm: j for j, lcm in enumerate(V2Dref(D, k, n, scheme), start=1)}


def V2D(D, k, n, vect, scheme="sparse"):
    coeffs = {}
    j = 0
    for level in cartesian((n + 1,) * D):
        if cutoff(scheme, level, n):
            continue
        ks = tuple(1 << max(0, level[q] - 2) for q in range(D))
        level_coeffs = {}
        for cell in cartesian(ks):
            cell_coeffs = {}
            for mode in cartesian((k,) * D):
                cell_coeffs[mode] = vect[j]
                j += 1
            level_coeffs[cell] = cell_coeffs
        coeffs[level] = level_coeffs
    return coeffs


def D2V(D, k, n, coeffs, scheme="sparse"):
    vect = []
    for level in cartesian((n + 1,) * D):
        if cutoff(scheme, level, n):
            continue
        ks = tuple(1 << max(0, level[q] - 2) for q in range(D))
        for cell in cartesian(ks):
            for mode in cartesian((k,) * D):
                vect.append(coeffs[level][cell][mode])
    return vect


def get_index_1D(k, l, c, m):
    """src/additional_tools.jl:18-20; for l = 1 the Julia shift by
    (l-2)%UInt wraps past the word size and yields 0."""
    shift = (1 << (l - 2)) if l >= 2 else 0
    return k * (shift + (c - 1)) + m
