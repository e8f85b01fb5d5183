"""Reader for AMPE's CALPHAD binary databases.

The reference reads its thermodynamic data through SAMRAI's input parser
(e.g. thermodynamic_data/calphadAuNi.dat:1-62): nested ``Name { ... }``
blocks of ``key = v1, v2, ...`` lines with ``//`` comments.  Species blocks
hold piecewise Gibbs energies
    G(T) = a + b T + c T ln T + sum_i d_i T^i     on [Tc_s, Tc_{s+1})
and ``LmixPhase*`` blocks hold Redlich-Kister coefficients
    L_k(T) = L_k[0] + L_k[1] T.
This module turns such a file (or its JSON image) into the ``g`` and ``L``
members of :class:`ampe_gb300.abi.Model`.
"""
import json
import re

from . import abi

_POWERS = {"d2": "d2", "d3": "d3", "d4": "d4", "d7": "d7", "dm1": "dm1", "dm9": "dm9"}


def parse_input_text(text):
    """Parse SAMRAI-style input text into nested dicts of float lists/strings."""
    text = re.sub(r"//[^\n]*", "", text)
    tokens = re.findall(r'"[^"]*"|[{}=,]|[^\s{}=,"]+', text)
    pos = 0

    def block():
        nonlocal pos
        out = {}
        while pos < len(tokens):
            tok = tokens[pos]
            if tok == "}":
                pos += 1
                return out
            name = tok
            pos += 1
            if tokens[pos] == "{":
                pos += 1
                out[name] = block()
                continue
            if tokens[pos] != "=":
                raise ValueError("expected '=' after %r" % name)
            pos += 1
            vals = [tokens[pos]]
            pos += 1
            while pos < len(tokens) and tokens[pos] == ",":
                vals.append(tokens[pos + 1])
                pos += 2
            conv = []
            for v in vals:
                if v.startswith('"'):
                    conv.append(v.strip('"'))
                else:
                    conv.append(float(v))
            out[name] = conv
        return out

    return block()


def database_from_text(text):
    """Return {'species': {'A': {'L': seg, 'S': seg}, 'B': ...}, 'L': {...}}."""
    tree = parse_input_text(text)
    db = {"species": {}, "Lmix": {}}
    for sp, key in (("A", "SpeciesA"), ("B", "SpeciesB")):
        node = tree[key]
        db["species"][sp] = {"name": node.get("name", [sp])[0]}
        for ph, pkey in (("L", "PhaseL"), ("S", "PhaseA")):
            p = node[pkey]
            seg = {"Tc": p["Tc"]}
            for coef in ("a", "b", "c") + tuple(_POWERS):
                if coef in p:
                    seg[coef] = p[coef]
            db["species"][sp][ph] = seg
    for ph, key in (("L", "LmixPhaseL"), ("S", "LmixPhaseA")):
        db["Lmix"][ph] = {k: v for k, v in tree.get(key, {}).items()}
    if "MobilityParameters" in tree:
        db["mobility"] = mobility_from_tree(tree["MobilityParameters"])
    return db


def mobility_from_tree(node):
    """The MobilityParameters block (CALPHADMobility::initialize,
    CALPHADMobility.cc:17-150; CompositionStrategyMobilities.cc:36-90) as
    {'0'|'1' (species): {'L'|'S' (phase): {'qA': [...], 'qB': [...],
    'q0AB': [...], ...}}}; keys absent from the block are absent here."""
    out = {}
    for s in ("0", "1"):
        sp = node["Species" + s]
        out[s] = {}
        for ph, key in (("L", "PhaseL"), ("S", "PhaseA")):
            out[s][ph] = {k: list(v) for k, v in sp[key].items()}
    return out


def mobility_struct(mob):
    """abi.Mobility from mobility_from_tree's dict: qA/qB take 2 or 4
    values (a0, a1[, a2, a3]); q<n>AB default to (0, 1) as in the
    reference."""
    mb = abi.Mobility()
    for si, s in enumerate(("0", "1")):
        for pi, ph in enumerate(("L", "S")):
            d = mob[s][ph]
            for ii, k in enumerate(("qA", "qB")):
                v = list(d[k])
                if len(v) not in (2, 4):
                    raise ValueError("%s of species %s, phase %s: %d values" % (k, s, ph, len(v)))
                v = v + [0.0] * (4 - len(v))
                for c in range(4):
                    mb.q[si][pi][ii][c] = v[c]
            for n in range(4):
                v = d.get("q%dAB" % n, [0.0, 1.0])
                mb.qq[si][pi][n][0] = v[0]
                mb.qq[si][pi][n][1] = v[1]
    return mb


def gterm_from_segments(seg):
    """Fill an abi.GTerm from one species/phase segment dict."""
    g = abi.GTerm()
    tc = list(seg["Tc"])
    nseg = len(tc) - 1
    if nseg > abi.MAX_TSEG:
        raise ValueError("too many temperature intervals: %d" % nseg)
    g.nseg = nseg
    for i, t in enumerate(tc):
        g.tc[i] = t
    for coef in ("a", "b", "c") + tuple(_POWERS):
        vals = seg.get(coef, [])
        arr = getattr(g, coef)
        for s in range(nseg):
            arr[s] = vals[s] if s < len(vals) else 0.0
    return g


def apply_database(model, db):
    """Set model.g and model.L (and model.mobility when the database has a
    MobilityParameters block) from a database dict (see database_from_text).
    Which diffusivities the model uses stays model.conc_diffusion's choice."""
    model.thermo = abi.THERMO_CALPHAD
    for si, sp in enumerate(("A", "B")):
        for pi, ph in enumerate(("L", "S")):
            model.g[si][pi] = gterm_from_segments(db["species"][sp][ph])
    for pi, ph in enumerate(("L", "S")):
        lm = db["Lmix"].get(ph, {})
        for k in range(4):
            v = lm.get("L%d" % k, [0.0, 0.0])
            model.L[pi][k][0] = v[0]
            model.L[pi][k][1] = v[1] if len(v) > 1 else 0.0
    if "mobility" in db:
        model.mobility = mobility_struct(db["mobility"])
    return model


def load_json(path):
    with open(path) as f:
        return json.load(f)
