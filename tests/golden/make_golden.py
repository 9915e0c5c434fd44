"""Extract the golden vectors the tests replay from the reference's committed
known-answer files, and copy the reference's committed circuit artifacts
(crates/constraints/tests/vectors/*.bin, the family circuits in their
postcard wire form) byte for byte into tests/golden/artifacts/.

The reference pins its hot path with text fixtures generated against
arkworks (ark-bn254 0.6) and Plonky3's Poseidon2; this script copies the
data lines the tests use into tests/golden/ (the Fq corpus keeps only its
base-field record kinds). Run it from the repository root, naming the root
of a checkout of the reference tree:

    python tests/golden/make_golden.py /path/to/apogee-vm

Every output file starts with a header naming its source file and the
selection applied.
"""
import os
import sys

SOURCES = {
    # name: (path inside the reference, line filter, max data lines (per kind) or None)
    "fr_kats.txt": ("crates/field/tests/vectors/fr_kats.txt", None, None),
    "fq_kats.txt": ("crates/curve/tests/vectors/fq_kats.txt", ("fq_ops", "fq_pow", "fq_bytes", "fq_u64"), None),
    "g1_kats.txt": ("crates/curve/tests/vectors/g1_kats.txt", None, None),
    "msm_kats.txt": ("crates/curve/tests/vectors/msm_kats.txt", None, None),
    "poly_kats.txt": ("crates/poly/tests/vectors/poly_kats.txt", None, None),
    "poseidon2_perm.txt": ("crates/transcript/tests/vectors/poseidon2_perm.txt", None, None),
    "transcript_cases.txt": ("crates/transcript/tests/vectors/transcript_cases.txt", None, None),
    "io_digest.txt": ("crates/transcript/tests/vectors/io_digest.txt", None, None),
    "evaluate_diff.txt": ("crates/poly/tests/vectors/evaluate_diff.txt", None, None),
    "g1_absorb_kats.txt": ("crates/pcs/tests/vectors/g1_absorb_kats.txt", None, None),
    "mercury_proof.txt": ("crates/pcs/tests/vectors/mercury_proof.txt", None, None),
    "mercury_batch.txt": ("crates/pcs/tests/vectors/mercury_batch.txt", None, None),
    "accumulator.txt": ("crates/pcs/tests/vectors/accumulator.txt", None, None),
    "pairing_kats.txt": ("crates/curve/tests/vectors/pairing_kats.txt", None, None),
    "g2_kats.txt": ("crates/curve/tests/vectors/g2_kats.txt", None, 200),
    "fq12_kats.txt": ("crates/curve/tests/vectors/fq12_kats.txt", ("fq12_ops", "fq12_final_exp"),
                      {"fq12_ops": 68, "fq12_final_exp": 20}),
}


ARTIFACTS = "crates/constraints/tests/vectors"


def copy_artifacts(ref_root: str, out_dir: str) -> None:
    dst = os.path.join(out_dir, "artifacts")
    os.makedirs(dst, exist_ok=True)
    src = os.path.join(ref_root, ARTIFACTS)
    for name in sorted(os.listdir(src)):
        if name.endswith(".bin"):
            with open(os.path.join(src, name), "rb") as f:
                data = f.read()
            with open(os.path.join(dst, name), "wb") as f:
                f.write(data)
            print(f"artifacts/{name}: {len(data)} bytes")


def main(ref_root: str) -> None:
    out_dir = os.path.dirname(os.path.abspath(__file__))
    copy_artifacts(ref_root, out_dir)
    for name, (rel, kinds, limit) in SOURCES.items():
        src = os.path.join(ref_root, rel)
        with open(src) as f:
            lines = f.read().splitlines()
        kept = []
        counts = {}
        for line in lines:
            if not line or line.startswith("#"):
                continue
            kind = line.split()[0]
            if kinds is not None and kind not in kinds:
                continue
            if limit is not None:
                counts[kind] = counts.get(kind, 0) + 1
                if counts[kind] > (limit[kind] if isinstance(limit, dict) else limit):
                    continue
            kept.append(line)
        if limit is None:
            sel = "all data lines"
        elif isinstance(limit, dict):
            sel = "first " + ", ".join(f"{v} {k}" for k, v in limit.items()) + " data lines"
        else:
            sel = f"first {limit} data lines of each record kind"
        if kinds is not None:
            sel += f" of kinds {', '.join(kinds)}"
        header = [f"# golden vectors from the reference's {rel}", f"# selection: {sel}"]
        with open(os.path.join(out_dir, name), "w") as f:
            f.write("\n".join(header + kept) + "\n")
        print(f"{name}: {len(kept)} lines")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <root of the reference checkout>")
    main(sys.argv[1])
