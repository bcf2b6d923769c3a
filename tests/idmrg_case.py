"""The engine's own H_eff at the last two-site step of a short run
(tests/golden/idmrg_*.npz, made by hamiltonian_vector_multiplication_idmrg,
dmrg_su2.cpp:543-664): shared by the oracle (CPU) and GPU tests."""
import numpy as np


def load(oracle, g):
    """Returns (psi Struct, psi, H psi in psi's layout, H psi blocks outside
    psi's layout, tensors {i: (Struct, data)}, terms, hl, hr).  terms =
    [(coef, [(L index, c)], [(R index, c)])]."""
    n = int(g["ntensors"])
    T = {}
    for i in range(n):
        d = g[f"t{i}_desc"]
        if int(d[0]) == 0:
            T[i] = None
            continue
        T[i] = (oracle.struct_from_desc(d, g[f"t{i}_flag"]), g[f"t{i}_x"])
    vs, vx = T[0]
    ys, yx = T[1]
    # H psi in psi's layout; whatever the reference put elsewhere must be zero
    y = oracle.to_layout(ys, yx, vs)
    outside = np.linalg.norm(yx) ** 2 - np.linalg.norm(y) ** 2
    ti, td = g["term_i"], g["term_d"]
    terms, q, r = [], 1, 0
    for _ in range(int(ti[0])):
        coef = float(td[r])
        r += 1
        sides = []
        for _side in range(2):
            k = int(ti[q])
            q += 1
            lst = []
            for _ in range(k):
                lst.append((int(ti[q]), float(td[r])))
                q += 1
                r += 1
            sides.append(lst)
        terms.append((coef, sides[0], sides[1]))
    return vs, vx, y, max(outside, 0.0), T, terms, T[2], T[3]


def combine_host(oracle, T, lst):
    """sum c * T[i] with the union of blocks (tensor_su2 operator+=)."""
    s0 = T[lst[0][0]][0]
    out = oracle.Struct(s0.bonds, s0.locspin)
    out.flag = np.zeros(s0.nten, np.int32)
    for i, _ in lst:
        out.flag = np.maximum(out.flag, T[i][0].flag).astype(np.int32)
    x = 0
    for i, c in lst:
        x = x + c * oracle.to_layout(T[i][0], T[i][1], out)
    return out, x
