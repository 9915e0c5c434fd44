"""The reference's circuit artifacts in the GKR entry points' own form.

A `constraints::CircuitArtifact` travels as postcard bytes (the wire form of
crates/constraints/src/wire.rs): a tuple per type, unsigned integers as LEB128
varints, `u8` and `bool` as one byte, strings and sequences prefixed with a
varint length, fixed arrays (an `Fr`, 32 canonical little-endian bytes) and
tuples as their elements in order, `Option` as a 0/1 byte before the value.
Per type (wire.rs):

* `PolyAddress` = (u8 tag, u32 a, u32 b): 0 M[a], 1 W[a], 2 S[a], 3 V[kind a],
  4 L{a}[b] (inner layer a, offset b), 5 scratch[a], 6 C{a}[b] (cached entry).
* `Coeff` = (u8 tag, u32 slot, Fr): 0 a literal, 1 a challenge slot.
* `GateDef` = (u8 tag, u32 split, [Coeff], [PolyAddress]) with tags 0 Linear,
  1 Product, 2 MaskIntoIdentity, 3 AffineProduct (split = left terms),
  4 TreeProduct, 5 Quadratic (split = linear terms), 6 TreeCross, and the
  coefficients / operands in GateDef::coefficients / operands order.
* `LayerSpec` = (halving, num_vars, width, [cached], [producing],
  [enforcing]); cached = (name, address, gate), producing = (relation, output,
  gate), enforcing = (relation, gate).
* `CircuitArtifact` = (format_version, coefficient_encoding, trace_vars,
  [M names], [W names], [S names], [(VirtualKind, name)], [LayerSpec],
  [relations], [lookups], [scratch], [outputs], ([padding Fr], bool)).

`to_circuit` resolves every address against its gate list the way the prover
reads it (layer 0 columns in M, W, S order, virtual tables by their position
in the artifact's list, cached entries by offset) and returns a
`circuits.Circuit`, whose `to_blob()` is the APGC blob of include/apogee_gpu.h.
The relations, lookups, scratch map and padding row are the constraint
system's and the verifier's; the GKR prover needs none of them.
"""
import circuits as C

FORMAT_VERSION = 1

# Wire gate tags -> the APGC shape numbers (circuits.py / include/apogee_gpu.h).
_SHAPE = {0: C.LINEAR, 1: C.PRODUCT, 2: C.MASK, 3: C.AFFINE, 4: C.TREE_PRODUCT, 5: C.QUADRATIC, 6: C.TREE_CROSS}


class ArtifactError(ValueError):
    """The bytes are not a circuit artifact this reader understands."""


class _Reader:
    def __init__(self, data: bytes):
        self.d = data
        self.i = 0

    def byte(self) -> int:
        if self.i >= len(self.d):
            raise ArtifactError("truncated artifact")
        b = self.d[self.i]
        self.i += 1
        return b

    def varint(self) -> int:
        v, shift = 0, 0
        while True:
            b = self.byte()
            v |= (b & 0x7F) << shift
            if b < 0x80:
                return v
            shift += 7
            if shift > 63:
                raise ArtifactError("varint too long")

    def boolean(self) -> bool:
        b = self.byte()
        if b > 1:
            raise ArtifactError("malformed bool")
        return b == 1

    def raw(self, n: int) -> bytes:
        if self.i + n > len(self.d):
            raise ArtifactError("truncated artifact")
        out = self.d[self.i:self.i + n]
        self.i += n
        return out

    def string(self) -> str:
        return self.raw(self.varint()).decode("utf-8")

    def seq(self, item):
        return [item() for _ in range(self.varint())]

    def fr(self) -> int:
        v = int.from_bytes(self.raw(32), "little")
        if v >= C.P_R:
            raise ArtifactError("non-canonical Fr")
        return v

    def address(self):
        return (self.byte(), self.varint(), self.varint())

    def coeff(self):
        tag, slot, v = self.byte(), self.varint(), self.fr()
        if tag == 0 and slot == 0:
            return ("lit", v)
        if tag == 1 and v == 0:
            return ("ch", slot)
        raise ArtifactError("malformed coefficient")

    def gate(self):
        tag, split = self.byte(), self.varint()
        coeffs = self.seq(self.coeff)
        ops = self.seq(self.address)
        return {"tag": tag, "split": split, "coeffs": coeffs, "ops": ops}

    def layer(self):
        halving, nv, width = self.boolean(), self.varint(), self.varint()
        cached = self.seq(lambda: (self.string(), self.address(), self.gate()))
        producing = self.seq(lambda: (self.varint(), self.address(), self.gate()))
        enforcing = self.seq(lambda: (self.varint(), self.gate()))
        return {"halving": halving, "num_vars": nv, "width": width, "cached": cached, "producing": producing,
                "enforcing": enforcing}

    def relation(self):
        name = self.string()
        out = self.varint() if self.boolean() else None
        return (name, out, self.gate())


def decode(data: bytes) -> dict:
    """The artifact's fields (gates as dicts of wire tag, split, coefficients
    and operands)."""
    r = _Reader(data)
    art = {"format_version": r.varint()}
    if art["format_version"] != FORMAT_VERSION:
        raise ArtifactError(f"format version {art['format_version']}")
    art["coefficient_encoding"] = r.varint()
    art["trace_vars"] = r.varint()
    art["memory"] = r.seq(r.string)
    art["witness"] = r.seq(r.string)
    art["setup"] = r.seq(r.string)
    art["virtuals"] = r.seq(lambda: (r.varint(), r.string()))
    art["layers"] = r.seq(r.layer)
    art["relations"] = r.seq(r.relation)
    art["lookups"] = r.seq(lambda: (r.string(), r.varint(), r.address(), r.seq(r.gate)))
    art["scratch"] = r.seq(lambda: (r.string(), r.address()))
    art["outputs"] = r.seq(r.address)
    art["padding"] = (r.seq(r.fr), r.boolean())
    if r.i != len(data):
        raise ArtifactError("trailing bytes")
    return art


def _operand(art, k, addr):
    """An address as gate list k reads it: (APGC source, index)."""
    tag, a, b = addr
    nm, nw = len(art["memory"]), len(art["witness"])
    if k == 0 and tag in (0, 1, 2):
        return C.col(a + (0 if tag == 0 else nm if tag == 1 else nm + nw))
    if tag == 4 and a == k and k > 0:
        return C.col(b)
    if tag == 3:
        kinds = [kind for kind, _ in art["virtuals"]]
        if a not in kinds:
            raise ArtifactError(f"virtual table {a} not declared")
        return C.virt(kinds.index(a))
    if tag == 6 and a == k:
        return C.cached(b)
    raise ArtifactError(f"address {addr} is not readable by gate list {k}")


def _gate(art, k, g):
    coeffs = [c[1] if c[0] == "lit" else ("ch", c[1]) for c in g["coeffs"]]
    ops = [_operand(art, k, a) for a in g["ops"]]
    shape = _SHAPE.get(g["tag"])
    if shape is None:
        raise ArtifactError(f"gate tag {g['tag']}")
    t = g["split"]
    if shape == C.LINEAR:
        return (shape, len(ops), 0, ops, coeffs)
    if shape == C.AFFINE:
        return (shape, t, len(ops) - t, ops, coeffs)
    if shape == C.QUADRATIC:
        return (shape, t, (len(ops) - t) // 2, ops, coeffs)
    return (shape, 0, 0, ops, coeffs)


def _signature(L):
    """A gate list's gates without their names, relation numbers or the
    index of the layer they read (so equal lists at different heights match)."""
    def ops(g):
        return tuple((t, b) if t in (4, 6) else (t, a, b) for t, a, b in g["ops"])

    def gates(es, gi):
        return [(e[gi]["tag"], e[gi]["split"], tuple(e[gi]["coeffs"]), ops(e[gi])) for e in es]

    return (L["halving"], L["width"], gates(L["cached"], 2), gates(L["producing"], 2), gates(L["enforcing"], 1))


def to_circuit(art: dict, trace_vars=None) -> C.Circuit:
    """The artifact's gate lists as an APGC circuit. With `trace_vars` below
    the artifact's, the same circuit over fewer rows: every list keeps its
    gates over `shift` fewer variables, and a product / fraction tree that
    halves down to one row (its identical halving lists at the top) loses
    its last `shift` levels, so the output map still names the top layer."""
    layers = art["layers"]
    shift = 0 if trace_vars is None else art["trace_vars"] - trace_vars
    if shift < 0:
        raise ArtifactError("cannot grow a circuit")
    if shift and min(L["num_vars"] for L in layers) >= shift:
        layers = [dict(L, num_vars=L["num_vars"] - shift) for L in layers]
    elif shift:
        top = layers[-shift:] if shift <= len(layers) else []
        keep = layers[:len(layers) - shift]
        if (len(top) != shift or not keep or not all(L["halving"] for L in top)
                or any(_signature(L) != _signature(keep[-1]) for L in top)):
            raise ArtifactError("the circuit's top is not a halving chain that can lose levels")
        if min(L["num_vars"] for L in keep) < shift:
            raise ArtifactError("too few rows for this circuit")
        layers = [dict(L, num_vars=L["num_vars"] - shift) for L in keep]
    n_committed = len(art["memory"]) + len(art["witness"]) + len(art["setup"])
    circ = C.Circuit(art["trace_vars"] - shift, n_committed, [kind for kind, _ in art["virtuals"]])
    for k, L in enumerate(layers):
        cac = [_gate(art, k, g) for _name, _addr, g in L["cached"]]
        prod = [_gate(art, k, g) for _rel, _out, g in L["producing"]]
        enf = [_gate(art, k, g) for _rel, g in L["enforcing"]]
        circ.add_layer(prod, cached=cac, enforcing=enf, halving=L["halving"])
        if circ.vars(k + 1) != L["num_vars"] or circ.width(k + 1) != L["width"]:
            raise ArtifactError(f"gate list {k}: stored shape does not match its gates")
    depth = len(art["layers"])
    outs = []
    for tag, a, b in art["outputs"]:
        if tag == 4 and a == depth and b < circ.width(circ.depth()):
            outs.append(b)
        elif depth == 0 and tag in (0, 1, 2):
            outs.append(_operand(art, 0, (tag, a, b))[1])
        else:
            raise ArtifactError("an output that is not a top-layer column")
    circ.outputs = outs
    return circ
