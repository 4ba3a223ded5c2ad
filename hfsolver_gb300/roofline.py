"""Algorithmic work units of the pipeline's rooflines, stated once.

These are the counts the measurements divide by, independent of how a kernel
executes them (a kernel that skips zero Hermite terms does fewer flops than it is
credited with; one that recomputes does more):

* ERIs: a fixed McMurchie-Davidson count per *primitive* shell quartet
  (la lb | lc ld), the same formula the library sums into `eri_flops`
  (`hfgpu_md_flops`):
      F = 30 + 3L + 2 C(L+4, 4) + 2 nc(lc) nc(ld) nH(Lp) nH(Lq)
          + 2 nc(la) nc(lb) nc(lc) nc(ld) nH(Lp),
  Lp = la + lb, Lq = lc + ld, L = Lp + Lq, nc(l) = (l+1)(l+2)/2 Cartesian
  components, nH(L) = (L+1)(L+2)(L+3)/6 Hermite functions up to L.
* Fock build: 12 flops (6 fused multiply-adds) and 8 bytes read per component
  quartet digested (J_ab, J_cd and the four exchange terms of one integral).
* AO->MO transform: the dense quarter transforms without permutational savings,
  2 o N^4 + 2 o v N^3 + 2 o^2 v N^2 + 2 o^2 v^2 N FP64-equivalent flops; the
  tensor-core path performs 21 bf16 products for each FP64 multiply-add
  (six 7-bit slices per operand, products of digit order <= 5).
* MBPT2 energy sum: 8 o^2 v^2 bytes (the (ia|jb) block read once).
"""
from math import comb

__all__ = ["ncart", "nherm", "md_flops", "fock_flops", "fock_bytes", "transform_flops", "tensor_flops",
           "mp2_sum_bytes", "SLICE_PRODUCTS"]

SLICE_PRODUCTS = 21  # bf16 products per FP64 multiply-add: slice pairs (i, j) with i + j <= 5


def ncart(l):
    """Cartesian components of angular momentum l."""
    return (l + 1) * (l + 2) // 2


def nherm(L):
    """Hermite Gaussians t + u + v <= L."""
    return (L + 1) * (L + 2) * (L + 3) // 6


def md_flops(la, lb, lc, ld):
    """FP64 flops credited to one primitive shell quartet (la lb | lc ld)."""
    Lp, Lq = la + lb, lc + ld
    L = Lp + Lq
    return (30 + 3 * L + 2 * comb(L + 4, 4) + 2 * ncart(lc) * ncart(ld) * nherm(Lp) * nherm(Lq)
            + 2 * ncart(la) * ncart(lb) * ncart(lc) * ncart(ld) * nherm(Lp))


def fock_flops(component_quartets):
    """Flops of one Fock build digesting this many component quartets."""
    return 12.0 * component_quartets


def fock_bytes(component_quartets):
    """Integral bytes one Fock build reads."""
    return 8.0 * component_quartets


def transform_flops(n, o, v):
    """FP64-equivalent flops of the four quarter transforms for (ia|jb)."""
    return 2.0 * o * n ** 4 + 2.0 * o * v * n ** 3 + 2.0 * o * o * v * n ** 2 + 2.0 * o * o * v * v * n


def tensor_flops(m, n, k):
    """bf16 tensor-pipe flops of one exactly sliced m x n x k FP64 product."""
    return 2.0 * SLICE_PRODUCTS * m * n * k


def mp2_sum_bytes(o, v):
    """Bytes of the (ia|jb) block the MBPT2 energy sum reads."""
    return 8.0 * o * o * v * v
