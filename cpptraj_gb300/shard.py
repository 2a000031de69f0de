"""Host-side partition of the all-pairs output across ranks.

Pairs are independent, so sharding needs no data-path collective: rank r
computes the output rows [row_begin, row_end) it owns through the row-range
arguments of gbr_allpairs and writes them at their offset in the shared
layout.  TRI rows (reference frames) shrink from n-1 elements to 0, so the
ranges are balanced by pair count; FULL rows (target frames) all hold n_ref
elements and are split evenly.
"""
from __future__ import annotations


def tri_elements_before(n: int, i: int) -> int:
    """Elements of the triangle stored before row i (calcTriIndex layout)."""
    return i * n - (i * (i + 1)) // 2


def tri_row_ranges(n: int, nranks: int):
    """Contiguous TRI row ranges with about equal pair counts, one per rank."""
    total = tri_elements_before(n, n)
    out, start = [], 0
    for r in range(nranks):
        target = (total * (r + 1)) // nranks
        end = start
        while end < n and tri_elements_before(n, end) < target:
            end += 1
        if r == nranks - 1:
            end = n
        out.append((start, end))
        start = end
    return out


def full_row_ranges(n_tgt: int, nranks: int):
    """Even split of FULL rows (target frames)."""
    return [((n_tgt * r) // nranks, (n_tgt * (r + 1)) // nranks) for r in range(nranks)]


def output_offset(n_ref: int, out_kind: int, row_begin: int) -> int:
    """Offset of row_begin's first element in the whole-matrix layout."""
    if out_kind == 0:
        return tri_elements_before(n_ref, row_begin)
    return row_begin * n_ref
