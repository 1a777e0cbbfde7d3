"""Extract the group-theoretical coupling-coefficient table into a data file.

The potential file format (``mlp.lammps``) stores regression coefficients
whose meaning is fixed by one particular table of rotational-invariant
coupling coefficients: the literal table in the reference package,
``src/USER-MLIP/mlipkk_gtinv_data.cpp`` (``l_array_all`` at :35,
``coeffs_all`` at :185, ``m_array_all`` at :12383).  A potential file is
only meaningful together with exactly that table (same irreps order, same
term order, same coefficient values), so this project carries it as data.

This script parses the three initializer lists from that source file as
text and writes ``gtinv_table.txt`` next to itself.  The decimal strings are
copied unchanged, so every coefficient parses to the same double as in the
reference build.

File format (whitespace separated, ``#`` starts a comment line)::

    <n_irreps>
    repeated n_irreps times:
        <order q> <l_1> ... <l_q> <n_terms>
        repeated n_terms times:
            <coefficient> <m_1> ... <m_q>

Run once, where the reference sources are available::

    python make_gtinv_table.py /path/to/reference/src/USER-MLIP/mlipkk_gtinv_data.cpp
"""
import os
import re
import sys


def _block(src, name):
    i = src.index(name + " =")
    j = src.index("{", i)
    depth = 0
    for k in range(j, len(src)):
        if src[k] == "{":
            depth += 1
        elif src[k] == "}":
            depth -= 1
            if depth == 0:
                return src[j:k + 1]
    raise ValueError("unterminated initializer for " + name)


def _nested(text):
    stack = [[]]
    for tok in re.findall(r"\{|\}|[-+0-9.eE]+", text):
        if tok == "{":
            stack.append([])
        elif tok == "}":
            done = stack.pop()
            stack[-1].append(done)
        else:
            stack[-1].append(tok)
    return stack[0][0]


def extract(src_path):
    src = open(src_path).read()
    l_all = _nested(_block(src, "l_array_all"))
    c_all = _nested(_block(src, "coeffs_all"))
    m_all = _nested(_block(src, "m_array_all"))
    if not (len(l_all) == len(c_all) == len(m_all)):
        raise ValueError("table arrays differ in length")
    out = ["# rotational-invariant coupling coefficients (irreps, terms)",
           "# extracted verbatim from mlipkk_gtinv_data.cpp by make_gtinv_table.py",
           str(len(l_all))]
    for ls, cs, ms in zip(l_all, c_all, m_all):
        if len(cs) != len(ms):
            raise ValueError("term count mismatch")
        out.append(" ".join([str(len(ls))] + ls + [str(len(cs))]))
        for c, m in zip(cs, ms):
            if len(m) != len(ls):
                raise ValueError("m list length mismatch")
            out.append(" ".join([c] + m))
    return "\n".join(out) + "\n"


def main():
    src = sys.argv[1] if len(sys.argv) > 1 else \
        "/root/reference/src/USER-MLIP/mlipkk_gtinv_data.cpp"
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "gtinv_table.txt")
    with open(dst, "w") as f:
        f.write(extract(src))
    print("wrote", dst)


if __name__ == "__main__":
    main()
