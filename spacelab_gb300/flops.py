"""Algorithmic work of one unordered pair of the reference's pass 2
(ColliderSingleCore.cpp:104-253), for roofline arithmetic.

Convention: every double add, subtract, multiply, divide and square root
counts as one flop; constant folds (Ha/6*64), negations, fabs, comparisons
and selects count zero; identical subexpressions are counted once (the
reference recomputes rVecab.norm() inside normalized(); it equals `dist`).
The counts are per UNORDERED pair, i.e. per evaluation the reference makes.
"""

# non-contact branch, :104-116, :205-227, :249-253
NONCONTACT = {
    "sumRaRb": 1,                 # R[A] + R[B]
    "rVecab": 3,                  # pos[B] - pos[A]
    "dist": 6,                    # 3 mul, 2 add, 1 sqrt
    "overlap": 1,
    "vdw_magnitude": 23,          # h2 1, 2Ra h 2, 2Rb h 2, S 2, 4RaRb 2, T 1, h+Ra+Rb 2,
                                  # S*S*T*T 3, quotient 1, *Ra^3 Rb^3 6, * quotient 1
    "normalized": 3,              # 3 div (norm shared with dist)
    "scale": 3,                   # magnitude * unit vector
    "acc_updates": 12,            # F/m[A] 3 div + 3 add, F/m[B] 3 div + 3 sub
}

# contact branch adds (:119-204) on top of sumRaRb, rVecab, dist, overlap,
# vdw_magnitude, normalized, scale and the acc updates
CONTACT_EXTRA = {
    "elastic": 2 + 3,             # -k*overlap*.5 (2 mul), * unit (3)
    "gravity": 4 + 3,             # G*mA*mB/(dist*dist): 2 mul, 1 mul, 1 div; * unit
    "elastic_norm": 6,
    "r_a": 6, "r_b": 6,           # (r*R)/sum
    "w_diff": 3, "d_vel": 3,
    "frame": 5 + 1 + 3 + 3 + 9 + 9 + 6,  # dot 5, dist^2 1, r/dd 3, dot*u 3, 2 crosses 9+9, 2x3 subs
    "rel_vel_mag": 6,
    "slide": 1 + 3 + 3,           # u_s*efm, frame/rvm, scale
    "w_diff_mag": 6,
    "roll": 9 + 6 + 1 + 3 + 3,    # cross, its norm, -u_r*efm, scale, divide
    "total_force": 9,             # three vector adds
    "torques": 3 + 9 + 3 + 9,     # s+q, cross, -s+q, cross
    "aacc_updates": 12,           # torque/moi 3 div + 3 add, twice
}

# write-step potential energy per pair, :195-203 / :231-239 (log counted as 1)
PE_NONCONTACT = 17
PE_CONTACT_EXTRA = 4              # + 0.5*k*overlap*overlap and the add

FLOPS_NONCONTACT = sum(NONCONTACT.values())
FLOPS_CONTACT = FLOPS_NONCONTACT + sum(CONTACT_EXTRA.values())


def pair_flops(pairs: int, contacts: int, write: bool = False) -> float:
    """Algorithmic flops of one pass 2 over `pairs` unordered pairs of which
    `contacts` are in contact."""
    nc = pairs - contacts
    f = nc * FLOPS_NONCONTACT + contacts * FLOPS_CONTACT
    if write:
        f += pairs * PE_NONCONTACT + contacts * PE_CONTACT_EXTRA
    return float(f)


# Bytes of HBM traffic the exact step's kernels need per sphere and per pair.
#   pair kernel: stores 2 x 24 B of force terms per unordered pair
#   row sums:    loads those 48 B per unordered pair (24 B per ordered pair)
PAIR_TERM_BYTES_WRITE = 48
PAIR_TERM_BYTES_READ = 48


# The FP64 work per pair of the mixed form with FP64 geometry and
# accumulation (SL_MODE_MIXED, sl_step_mixed64.cu), which bounds it: the
# subtraction pos[B] - pos[A] (3 adds) and the two spheres' FP64 force sums
# (3 + 3 adds).  Close pairs add their FP64 |r|^2, gap, sqrt and overlap,
# O(N) of the O(N^2) pairs.
MIXED64_FP64_OPS_PER_PAIR = 9
