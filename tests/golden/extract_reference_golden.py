"""Extract the literal golden values of the reference's own tests into reference_golden.json.

Reads (as text, never executes) the Julia test files of fdDGAsolver.jl and records the numbers
that pin the parquet-iteration path:

* test/test_siam_scPA.jl:28-31, :60-63  -- Σ at 4 fermionic and γa/γp/γt K1 at 4 bosonic-axis points
* test/test_siam_fdPA.jl:179            -- Σ(πT) of the fdPA solve from a Vertex-valued reference
* test/test_hubbard.jl:84-88            -- Hubbard occupations

Usage: python tests/golden/extract_reference_golden.py <reference_root>
The reference checkout is read only here; tests use the committed JSON.
"""
import json
import os
import re
import sys

NUM = r"[-+]?\d+\.\d+(?:e[-+]?\d+)?"
CNUM = rf"{NUM}(?:\s*[-+]\s*{NUM}im)?"


def parse_complex(tok: str) -> list:
    tok = tok.replace(" ", "")
    m = re.fullmatch(rf"({NUM})(?:([-+]{NUM})im)?", tok)
    if not m:
        raise ValueError(tok)
    return [float(m.group(1)), float(m.group(2)) if m.group(2) else 0.0]


def vec_after(text: str, anchor: str, start: int = 0):
    i = text.index(anchor, start)
    j = text.index("[", text.index("≈", i))
    k = text.index("]", j)
    toks = [t.strip() for t in text[j + 1:k].split(",")]
    return [parse_complex(t) for t in toks], k


def main(root: str) -> dict:
    out = {"source": "fdDGAsolver.jl test files (literal values)"}
    scpa = open(os.path.join(root, "test", "test_siam_scPA.jl"), encoding="utf-8").read()
    pos = 0
    for case in ("half_filling", "doped"):
        rec = {}
        for key, anchor in (("Sigma", "S.Σ.("), ("a", "S.F.γa.K1.("), ("p", "S.F.γp.K1.("), ("t", "S.F.γt.K1.(")):
            rec[key], pos = vec_after(scpa, anchor, pos)
        out[f"siam_scPA_{case}"] = rec
    out["siam_scPA_half_filling"]["params"] = dict(T=0.1, U=1.0, e=0.0, Delta="pi/5", D=10.0, nG=36, nK1=24,
                                                   nK2=[6, 6], nK3=[6, 6], sigma_n=[-2, -1, 0, 1],
                                                   k1_x="2*pi*T*-2 + [0,1,2,3]")
    out["siam_scPA_doped"]["params"] = dict(T=0.1, U=1.0, e=0.5, Delta="pi/5", D=10.0, nG=36, nK1=24,
                                            nK2=[7, 6], nK3=[7, 6], sigma_n=[-2, -1, 0, 1],
                                            k1_x="2*pi*T*-2 + [0,1,2,3]")
    fdpa = open(os.path.join(root, "test", "test_siam_fdPA.jl"), encoding="utf-8").read()
    m = re.search(rf"S_fd2\.Σ\(π\*T\)\s*≈\s*({CNUM})", fdpa)
    out["siam_fdPA_sigma_piT"] = {"value": parse_complex(m.group(1)),
                                  "params": dict(T=0.1, U=1.0, ref=dict(e=-0.3, Delta="pi/3", D=10.0, nmax=12),
                                                 target=dict(e=0.5, Delta="pi/5", D=20.0, nmax=8))}
    hub = open(os.path.join(root, "test", "test_hubbard.jl"), encoding="utf-8").read()
    occ = []
    for mm in re.finditer(rf"compute_occupation\(hubbard_bare_Green\(mG, mK; t1=1\., μ=([-+]?\d+\.\d*)\)\)\s*≈\s*(.+)", hub):
        mu = float(mm.group(1))
        rhs = mm.group(2).strip()
        val = eval(rhs, {"__builtins__": {}}, {})  # plain arithmetic like "1 - 0.0502..."
        occ.append([mu, float(val)])
    out["hubbard_occupation"] = {"values": occ, "params": dict(T=0.5, nG=20, L=8, t1=1.0)}
    return out


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: extract_reference_golden.py <path of the fdDGAsolver.jl checkout>")
    data = main(sys.argv[1])
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "reference_golden.json"), "w") as f:
        json.dump(data, f, indent=1)
    print(json.dumps(data)[:400])
