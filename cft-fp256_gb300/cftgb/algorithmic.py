"""The algorithmic work of one element, frozen in one place: what the
roofline numbers of the benchmark divide by.

L is the number of 32-bit limbs of a format's encoding (1, 2, 4, 8 for
binary32/64/128/256). Integer operations an element:

  FMA, MUL   2 L^2 multiply halves (mad.lo / mad.hi) for the exact product,
             plus 8 L simple operations to align, add, normalise and round
  ADD, SUB   8 L simple operations (no product)
  DIV        2 L (L + 1) multiply halves (schoolbook long division, Knuth
             Algorithm D) plus 8 L
  SQRT       L (L + 1) multiply halves plus 8 L

Bytes an element: (operands read + 1) x element size (FMA reads a, b, c;
ADD/SUB read a, c; MUL and DIV read a, b; SQRT reads a).
"""

LIMBS = {0: 1, 1: 2, 2: 4, 3: 8}
READS = {"fma": 3, "add": 2, "sub": 2, "mul": 2, "div": 2, "sqrt": 1}


def int_ops(fmt, op):
    L = LIMBS[fmt]
    if op in ("fma", "mul"):
        return 2 * L * L + 8 * L
    if op in ("add", "sub"):
        return 8 * L
    if op == "div":
        return 2 * L * (L + 1) + 8 * L
    if op == "sqrt":
        return L * (L + 1) + 8 * L
    raise KeyError(op)


def bytes_per_element(fmt, op):
    return (READS[op] + 1) * 4 * LIMBS[fmt]


def int_issue_peak_tops(sm_count=152, sm_mhz=2070.0):
    """Nominal integer issue rate: SMs x 4 schedulers x 32 lanes x clock, in
    tera-operations a second (no measured integer peak exists; this is the
    upper bound one instruction a lane a clock sets)."""
    return sm_count * 4 * 32 * sm_mhz * 1e6 / 1e12
