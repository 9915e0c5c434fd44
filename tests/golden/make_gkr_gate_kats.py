"""Write gkr_gate_kats.json: the gate kernel's literal known answers.

The cases restate crates/gkr/tests/kernel.rs of the reference (the tests
`linear`, `product`, `mask_into_identity`, `affine_product` and `quadratic`):
each gate variant with literal coefficients other than 0 and +-1, the
challenge coefficient gamma in slot TOY (= 0), and a nonzero constant on
every side that has one; the expected value is the arithmetic that file
writes out by hand, and the `not` values are the mutants it rules out (a
dropped coefficient, a constant taken from the wrong side). The two tree
gates, which kernel.rs leaves to the toy circuit, follow eval_gate's own
formulas (crates/gkr-verify/src/lib.rs:192-196): TreeProduct x(.,0) x(.,1),
TreeCross p(.,0) q(.,1) + p(.,1) q(.,0).

A case's operands are column indices; `columns` holds one value per column
for a row-wise gate and the pair (child 0, child 1) per column for a tree
gate. Gates use the APGC tuple of circuits.py: [shape, split1, split2,
operand columns, coefficients], a coefficient being an int or ["ch", slot].

Usage: python make_gkr_gate_kats.py  (writes next to this script)
"""
import json
import os

P = 21888242871839275222246405745257275088548364400416034343698204186575808495617
LINEAR, PRODUCT, MASK, AFFINE, TREE_PRODUCT, TREE_CROSS, QUADRATIC = range(7)
TOY = 0  # constants::challenge_slot::TOY
GAMMA = 0x9E3779B97F4A7C15 * 0x0123456789ABCDEF % P
CH = ["ch", TOY]


def case(name, gate, columns, expect, not_=()):
    return {"name": name, "gate": gate, "columns": columns, "expect": expect % P, "not": [x % P for x in not_]}


def cases():
    g = GAMMA
    out = []
    # linear: sum c_i x_i + c_0 with literals 2 and 5, a challenge coefficient, constant 7.
    out.append(case("linear", [LINEAR, 3, 0, [0, 1, 2], [2, 5, CH, 7]], [11, 13, 17],
                    2 * 11 + 5 * 13 + 7 + g * 17))
    # ... then a challenge as the constant.
    out.append(case("linear/challenge-constant", [LINEAR, 1, 0, [0], [3, CH]], [11], 33 + g))
    # product: c x y with c = 3 (not x y: the coefficient is not dropped), then c = gamma.
    out.append(case("product", [PRODUCT, 0, 0, [0, 1], [3]], [11, 13], 3 * 11 * 13, not_=[11 * 13]))
    out.append(case("product/challenge", [PRODUCT, 0, 0, [0, 1], [CH]], [11, 13], g * 143))
    # mask_into_identity: x m + (1 - m), under mask 1, mask 0 and off the bits.
    out.append(case("mask/1", [MASK, 0, 0, [0, 1], []], [11, 1], 11))
    out.append(case("mask/0", [MASK, 0, 0, [0, 1], []], [11, 0], 1))
    out.append(case("mask/5", [MASK, 0, 0, [0, 1], []], [11, 5], 11 * 5 + 1 - 5))
    # affine_product: (2 x0 + gamma x1 + 3)(5 x2 + 7); the right constant is its
    # own and the left constant is kept.
    left = 2 * 11 + 3 + g * 13
    out.append(case("affine", [AFFINE, 2, 1, [0, 1, 2], [2, CH, 3, 5, 7]], [11, 13, 17], left * (5 * 17 + 7),
                    not_=[left * (5 * 17 + 3), (2 * 11 + g * 13) * (5 * 17 + 7)]))
    # ... then a challenge as the right constant.
    out.append(case("affine/challenge-constant", [AFFINE, 1, 1, [0, 1], [2, 3, 5, CH]], [11, 17],
                    (2 * 11 + 3) * (5 * 17 + g)))
    # quadratic: 7 + 2 x0 + gamma x1 + 3 x2 x3 + gamma x4 x5 + 5 x0 x2, one operand read twice.
    products = 3 * 17 * 19 + 5 * 11 * 17 + g * 23 * 29
    out.append(case("quadratic", [QUADRATIC, 2, 3, [0, 1, 2, 3, 4, 5, 0, 2], [7, 2, CH, 3, CH, 5]],
                    [11, 13, 17, 19, 23, 29], 7 + 2 * 11 + g * 13 + products,
                    not_=[2 * 11 + g * 13 + products,
                          7 + 2 * 11 + 17 * 19 + 5 * 11 * 17 + g * 13 + g * 23 * 29]))
    out.append(case("quadratic/no-linear", [QUADRATIC, 0, 1, [0, 1], [CH, 3]], [11, 13], g + 429))
    out.append(case("quadratic/no-products", [QUADRATIC, 1, 0, [0], [7, 2]], [11], 29))
    out.append(case("quadratic/constant-only", [QUADRATIC, 0, 0, [], [7]], [], 7))
    # The tree gates at two children per column.
    out.append(case("tree-product", [TREE_PRODUCT, 0, 0, [0], []], [[11, 13]], 11 * 13))
    out.append(case("tree-cross", [TREE_CROSS, 0, 0, [0, 1], []], [[11, 13], [17, 19]], 11 * 19 + 13 * 17,
                    not_=[11 * 17 + 13 * 19]))
    out.append(case("tree-cross/same", [TREE_CROSS, 0, 0, [1, 1], []], [[11, 13], [17, 19]], 2 * 17 * 19))
    return out


def main():
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "gkr_gate_kats.json"), "w") as f:
        json.dump({"gamma": GAMMA, "slot": TOY, "cases": cases()}, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
