"""Patch a scratch COPY of the reference sources so GCC 13 can build them.

ORACLE / TEST INFRASTRUCTURE ONLY.  Never run on /root/reference itself: the
copy lives under /tmp and nothing of it enters this repository.

Eleven functions of the reference return a value type but fall off their end
without a return statement.  GCC 13 treats that as unreachable code (a trap at
-O0, a jump into the next function at -O2).  Their return values are never used
by the callers, so a plain `return` of the natural value is added before the
closing brace.  Each site is checked to still be a lone `}` before patching.

One test hook: the Lanczos length of the warm-up, a constant 5 in
lanczos_solve_eigenvector_idmrg (dmrg_su2.cpp:530), is read from the global
su2ref_idmrg_mlanc (defined in blas_shim.c, default 5, so the engine is
unchanged unless a test sets it).  A warm-up with five Lanczos vectors from
the uniform start vector stops near an invariant subspace and follows
rounding noise; with enough vectors to converge its result is a property of
the model, which is what the warm-up fixtures of the larger lattices pin.

A second hook adds the -seed option of the parity runs: the warm-up's start
vector (dmrg_su2_omp.cpp:79) is random_initialize_tensor when the global
su2ref_seeded is set (blas_shim.c su2ref_set_seed, which also seeds the
generator with initran), else the engine's own initialize_input_vector.
"""
import sys
from pathlib import Path

SITES = {
    # tensor& tensor::contract_dmrg_*  (tensor_dmrg_src.cpp) -> return *this
    "tensor_dmrg_src.cpp": [(101, "return *this;"), (166, "return *this;"),
                            (210, "return *this;"), (236, "return *this;"),
                            (272, "return *this;"), (360, "return *this;"),
                            (418, "return *this;"), (473, "return *this;")],
    # tensor_su2& operator=(double) -> *this ; int svd(...) -> 0
    "tensor_su2.cpp": [(103, "return *this;"), (1616, "return 0;"), (1758, "return 0;")],
}

# (file, line, expected text, replacement)
HOOKS = [("dmrg_su2.cpp", 530, "  int mlanc=5,nele1,nele2;",
          "  extern int su2ref_idmrg_mlanc;\n  int mlanc=su2ref_idmrg_mlanc,nele1,nele2;"),
         ("dmrg_su2_omp.cpp", 79, "      vec.initialize_input_vector();",
          "      { extern int su2ref_seeded; if (su2ref_seeded) vec.random_initialize_tensor(); "
          "else vec.initialize_input_vector(); }")]


def main(workdir: str) -> None:
    root = Path(workdir)
    for name, sites in SITES.items():
        path = root / name
        lines = path.read_text().split("\n")
        for lineno, stmt in sites:
            idx = lineno - 1
            if lines[idx].strip() != "}":
                raise SystemExit(f"{name}:{lineno}: expected a lone '}}', found {lines[idx]!r}")
            lines[idx] = "  " + stmt + "\n}"
        path.write_text("\n".join(lines))
    for name, lineno, want, repl in HOOKS:
        path = root / name
        lines = path.read_text().split("\n")
        if lines[lineno - 1].rstrip() != want:
            raise SystemExit(f"{name}:{lineno}: expected {want!r}, found {lines[lineno - 1]!r}")
        lines[lineno - 1] = repl
        path.write_text("\n".join(lines))


if __name__ == "__main__":
    main(sys.argv[1])
