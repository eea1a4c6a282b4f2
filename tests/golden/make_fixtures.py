"""Generate tests/golden/*.json from the reference checkout (run once, here; the output is committed).

Reads the reference's flat UPPAAL benchmark models (benchmarks/models/xml/<family><n>.xml and the
toy models under tests/models) together with its recorded verdict tables
(tests/uppaal-differential/round*.txt, each row a (model, query) pair on which HORA and UPPAAL
verifyta 5.0.0 agreed) and the recorded explored-state counts
(tests/models/urgent-chan/BASELINE-d4fb785.txt), and writes:

  tests/golden/models/<name>.json   the network in this repo's JSON form (ptctcl_gb300.model)
  tests/golden/verdicts.json        [{"model", "formula", "kind", "p", "q", "holds"}]

Only the flat subset of the modelling language is converted: clock / bounded-int / channel
declarations, location invariants, `var OP const` and clock guards joined by `&&`, `clock = 0`
resets, `var = const` updates and one synchronisation per edge -- exactly what the engine's
descriptor holds. `E[] psi` is kept when psi is a conjunction; `A<> phi` (= not E[] not phi) when
phi is a single atom, whose negation is again a conjunction. Models or formulas outside it
(functions, arrays, disjunctions) are skipped and listed on stdout.

Usage:  python tests/golden/make_fixtures.py [/path/to/reference]
"""
from __future__ import annotations

import json
import os
import re
import sys
import xml.etree.ElementTree as ET

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from ptctcl_gb300.model import (Network, Process, Location, Edge, IntVar, Pred, clock_atom,  # noqa: E402
                                IOP, CHAN_BROADCAST, CHAN_URGENT, query_to_json,
                                Q_REACH, Q_DEADLOCK, Q_LEADSTO, Q_EG)


class Unsupported(Exception):
    pass


ATOM = re.compile(r"^\s*([A-Za-z_]\w*)\s*(<=|>=|==|!=|<|>)\s*(-?\d+)\s*$")


def parse_decls(text: str, clocks, ints, chans):
    text = re.sub(r"//[^\n]*", "", text)
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    for stmt in text.split(";"):
        s = stmt.strip()
        if not s:
            continue
        if s.startswith("clock"):
            clocks.extend(x.strip() for x in s[5:].split(","))
            continue
        m = re.match(r"^(urgent\s+)?(broadcast\s+)?chan\s+(.*)$", s)
        if m:
            fl = (CHAN_URGENT if m.group(1) else 0) | (CHAN_BROADCAST if m.group(2) else 0)
            chans.extend((x.strip(), fl) for x in m.group(3).split(","))
            continue
        m = re.match(r"^int\s*\[\s*(-?\d+)\s*,\s*(-?\d+)\s*\]\s*(.*)$", s)
        if m:
            lo, hi = int(m.group(1)), int(m.group(2))
            for v in m.group(3).split(","):
                v = v.strip()
                init = 0 if lo <= 0 <= hi else lo
                if "=" in v:
                    v, iv = v.split("=")
                    v, init = v.strip(), int(iv)
                if "[" in v:
                    raise Unsupported("array")
                ints.append(IntVar(v, lo, hi, init))
            continue
        raise Unsupported(f"declaration: {s[:40]}")


def parse_guard(text, clocks, ivars, allow_ints=True):
    cons, iatoms = [], []
    if text is None or not text.strip():
        return cons, iatoms
    for atom in re.split(r"&&|\band\b", text):
        m = ATOM.match(atom)
        if not m:
            raise Unsupported(f"guard atom: {atom.strip()}")
        name, op, v = m.group(1), m.group(2), int(m.group(3))
        if name in clocks:
            x = clocks.index(name) + 1
            if op == "==":
                cons += [clock_atom(x, "<=", v), clock_atom(x, ">=", v)]
            elif op == "!=":
                raise Unsupported("clock !=")
            else:
                cons.append(clock_atom(x, op, v))
        elif name in ivars and allow_ints:
            iatoms.append((ivars.index(name), IOP[op], v))
        else:
            raise Unsupported(f"name {name}")
    return cons, iatoms


def load_flat(path: str) -> Network:
    root = ET.parse(path).getroot()
    clocks, ints, chans = [], [], []
    decl = root.find("declaration")
    if decl is not None and decl.text:
        parse_decls(decl.text, clocks, ints, chans)
    ivars = [v.name for v in ints]
    cnames = [c for c, _ in chans]
    templates = {}
    for t in root.findall("template"):
        name = t.find("name").text.strip()
        if t.find("parameter") is not None or t.find("declaration") is not None:
            raise Unsupported("template parameters/locals")
        ids, locs = {}, []
        for l in t.findall("location"):
            nm = l.find("name")
            lname = nm.text.strip() if nm is not None else l.get("id")
            inv = []
            for lab in l.findall("label"):
                if lab.get("kind") == "invariant":
                    c, ia = parse_guard(lab.text, clocks, ivars, allow_ints=False)
                    inv += c
            ids[l.get("id")] = len(locs)
            locs.append(Location(lname, inv, l.find("urgent") is not None, l.find("committed") is not None))
        init = ids[t.find("init").get("ref")]
        edges = []
        for tr in t.findall("transition"):
            e = Edge(ids[tr.find("source").get("ref")], ids[tr.find("target").get("ref")])
            for lab in tr.findall("label"):
                k, txt = lab.get("kind"), (lab.text or "").strip()
                if k == "guard":
                    e.guard, e.iguard = parse_guard(txt, clocks, ivars)
                elif k == "synchronisation":
                    m = re.match(r"^([A-Za-z_]\w*)\s*([!?])$", txt)
                    if not m or m.group(1) not in cnames:
                        raise Unsupported(f"sync {txt}")
                    e.chan, e.dir = cnames.index(m.group(1)), 1 if m.group(2) == "!" else -1
                elif k == "assignment":
                    for a in txt.split(","):
                        a = a.strip()
                        if not a:
                            continue
                        m = re.match(r"^([A-Za-z_]\w*)\s*:?=\s*(-?\d+)$", a)
                        if not m:
                            raise Unsupported(f"assignment {a}")
                        nm, v = m.group(1), int(m.group(2))
                        if nm in clocks:
                            if v != 0:
                                raise Unsupported("clock := nonzero")
                            e.resets.append(clocks.index(nm) + 1)
                        elif nm in ivars:
                            e.iupd.append((ivars.index(nm), v))
                        else:
                            raise Unsupported(f"assign to {nm}")
                elif k in ("select", "probability", "comments", "testcode"):
                    if k == "select":
                        raise Unsupported("select")
            edges.append(e)
        templates[name] = (locs, edges, init)
    sysline = root.find("system").text
    m = re.search(r"system\s+([^;]*);", sysline)
    procs = []
    for pn in m.group(1).split(","):
        pn = pn.strip()
        if pn not in templates:
            raise Unsupported(f"instantiation {pn}")
        locs, edges, init = templates[pn]
        nm = pn if sum(1 for p in procs if p.name.split("#")[0] == pn) == 0 else f"{pn}#{len(procs)}"
        procs.append(Process(nm, locs, edges, init))
    if len({p.name for p in procs}) != len(procs):
        raise Unsupported("duplicate process names")
    return Network(len(clocks), procs, ints, chans, ["0"] + clocks)


NEG_OP = {"<": ">=", "<=": ">", ">": "<=", ">=": "<", "==": "!=", "!=": "=="}


def parse_conj(text, net: Network, negate: bool = False, allow_neg: bool = False):
    """Conjunction of Proc.Loc, int and clock atoms -> Pred; with allow_neg also !Proc.Loc / negated
    atoms (the E[] route's restriction takes them). With negate, `text` must be a single atom and
    the Pred is its negation. Raises Unsupported otherwise."""
    p = Pred()
    text = text.strip()
    while text.startswith("(") and text.endswith(")"):
        text = text[1:-1].strip()
    atoms = [a.strip() for a in re.split(r"&&|\band\b", text)]
    if negate and len(atoms) != 1:
        raise Unsupported("negated conjunction")
    for atom in atoms:
        neg = negate
        m = re.match(r"^(?:!|not\s+)\s*(.*)$", atom)
        if m:
            if not allow_neg:
                raise Unsupported("negation")
            atom, neg = m.group(1).strip(), not neg
        m = re.match(r"^([A-Za-z_]\w*)\.([A-Za-z_]\w*)$", atom)
        if m:
            proc, loc = net.loc_index(m.group(1), m.group(2))
            p.loc_req.append((proc, -loc - 1) if neg else (proc, loc))   # negative: any other location
            continue
        m = ATOM.match(atom)
        if not m:
            raise Unsupported(f"atom {atom}")
        name, op, v = m.group(1), m.group(2), int(m.group(3))
        if neg:
            op = NEG_OP[op]
        cl = net.clock_names[1:]
        if name in cl:
            x = cl.index(name) + 1
            if op == "==":
                p.clk_cond += [clock_atom(x, "<=", v), clock_atom(x, ">=", v)]
            elif op == "!=":
                raise Unsupported("clock !=")
            else:
                p.clk_cond.append(clock_atom(x, op, v))
        elif name in [i.name for i in net.ints]:
            p.int_cond.append(([i.name for i in net.ints].index(name), IOP[op], v))
        else:
            raise Unsupported(f"name {name}")
    return p


def split_or(text: str):
    """Top-level `||` / `or` terms of a formula body (parentheses respected), outer parentheses
    around the whole body removed first."""
    text = text.strip()
    while text.startswith("(") and text.endswith(")"):
        depth, whole = 0, True
        for i, ch in enumerate(text):
            depth += ch == "("
            depth -= ch == ")"
            if depth == 0 and i < len(text) - 1:
                whole = False
                break
        if not whole:
            break
        text = text[1:-1].strip()
    terms, depth, cur, i = [], 0, "", 0
    while i < len(text):
        ch = text[i]
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if depth == 0 and text.startswith("||", i):
            terms.append(cur); cur = ""; i += 2; continue
        if depth == 0 and re.match(r"\bor\b", text[i:i + 3]) and (i == 0 or text[i - 1] == " "):
            terms.append(cur); cur = ""; i += 2; continue
        cur += ch
        i += 1
    terms.append(cur)
    return [t.strip() for t in terms if t.strip()]


def parse_formula_dnf(f: str, net: Network):
    """A formula whose top-level operand is a disjunction, lowered to several engine queries the
    binding combines: E<> (t1 || t2) = any E<> ti; A[] not (t1 || t2) = not any E<> ti;
    (p1 || p2) --> q = all pi --> q; A<> (a1 || a2) with single-atom terms = not E[] (!a1 && !a2).
    -> (terms [(kind, p, q)], combine "any" | "all", negate)."""
    f = f.strip()
    if f.startswith("E<>"):
        return [(Q_REACH, parse_conj(t, net), Pred()) for t in split_or(f[3:])], "any", False
    if f.startswith("A[]"):
        body = f[3:].strip()
        m = re.match(r"^(?:not|!)\s*\((.*)\)$", body)
        if not m:
            raise Unsupported("A[] form")
        return [(Q_REACH, parse_conj(t, net), Pred()) for t in split_or(m.group(1))], "any", True
    if f.startswith("A<>"):
        terms = split_or(f[3:])
        p = Pred()
        for t in terms:
            a = parse_conj(t, net, negate=True, allow_neg=True)
            p.loc_req += a.loc_req; p.int_cond += a.int_cond; p.clk_cond += a.clk_cond
        return [(Q_EG, p, Pred())], "any", True
    if "-->" in f:
        a, b = f.split("-->")
        if "!" in b or "||" in b or re.search(r"\bor\b", b):
            raise Unsupported("disjunctive or negated q")
        q = parse_conj(b, net)
        return [(Q_LEADSTO, parse_conj(t, net), q) for t in split_or(a)], "all", False
    raise Unsupported("formula")


def parse_formula(f: str, net: Network):
    """-> (kind, p, q, negate) where the verdict 'satisfied' = (engine result) xor negate."""
    f = f.strip()
    if "||" in f or re.search(r"\bor\b", f):
        raise Unsupported("formula form")
    if f.startswith("E[]"):
        return Q_EG, parse_conj(f[3:], net, allow_neg=True), Pred(), False
    if f.startswith("A<>"):
        return Q_EG, parse_conj(f[3:], net, negate=True, allow_neg=True), Pred(), True
    if f == "A[] not deadlock":
        return Q_DEADLOCK, Pred(), Pred(), True
    if f.startswith("E<>"):
        return Q_REACH, parse_conj(f[3:], net), Pred(), False
    if f.startswith("A[]"):
        body = f[3:].strip()
        m = re.match(r"^(?:not|!)\s*\((.*)\)$", body)
        if not m:
            raise Unsupported("A[] form")
        return Q_REACH, parse_conj(m.group(1), net), Pred(), True
    if "-->" in f:
        a, b = f.split("-->")
        if "!" in b:
            raise Unsupported("negation")
        return Q_LEADSTO, parse_conj(a, net), parse_conj(b, net), False
    raise Unsupported("formula")


def find_model(ref: str, name: str):
    name = name if name.endswith(".xml") else name + ".xml"
    for d in ("benchmarks/models/xml", "tests/models", "tests/models/urgent-chan",
              "tests/models/clock-liveness", "tests/liveness/refinement", "tests/liveness"):
        p = os.path.join(ref, d, name)
        if os.path.exists(p):
            return p
    return None


def main(ref: str):
    out_models = os.path.join(HERE, "models")
    os.makedirs(out_models, exist_ok=True)
    rows, skipped, nets, dnf_rows = [], [], {}, []
    tables = sorted(f for f in os.listdir(os.path.join(ref, "tests/uppaal-differential")) if f.endswith(".txt"))
    for tab in tables:
        for line in open(os.path.join(ref, "tests/uppaal-differential", tab)):
            cols = [c.strip() for c in line.split("|", 3)]
            if len(cols) < 4 or cols[0] != "ok":
                continue
            v = cols[1].split()
            if len(v) != 2 or v[0] != v[1] or v[0] not in ("SAT", "NOT"):
                continue
            mname, formula = cols[2], cols[3]
            key = mname.replace(".xml", "")
            try:
                if key not in nets:
                    path = find_model(ref, mname)
                    if path is None:
                        raise Unsupported("model file not found")
                    nets[key] = load_flat(path)
                net = nets[key]
                if net is None:
                    raise Unsupported("model not convertible")
                if "||" in formula or re.search(r"\bor\b", formula):
                    terms, combine, neg = parse_formula_dnf(formula, net)
                    sat = v[0] == "SAT"
                    dnf_rows.append({"model": key, "formula": formula, "table": tab, "combine": combine,
                                     "terms": [query_to_json(k_, p_, q_) for k_, p_, q_ in terms],
                                     "result": (not sat) if neg else sat})
                    continue
                kind, p, q, neg = parse_formula(formula, net)
            except (Unsupported, KeyError) as e:
                skipped.append((tab, mname, formula, str(e)))
                nets.setdefault(key, None)
                continue
            sat = v[0] == "SAT"
            # engine result convention: reach -> reachable; deadlock -> deadlock reachable; leadsto -> holds;
            # E[] psi -> holds (A<> phi is run as E[] not phi)
            result = (not sat) if neg else sat
            rows.append({"model": key, "formula": formula, "table": tab,
                         "query": query_to_json(kind, p, q), "result": result})
    # explored-state counts recorded by the reference for the deadlock route (informational)
    for key, net in nets.items():
        if net is not None:
            with open(os.path.join(out_models, key + ".json"), "w") as fh:
                fh.write(net.dumps())
    seen, uniq = set(), []
    for r in rows:
        k = (r["model"], r["formula"])
        if k not in seen:
            seen.add(k)
            uniq.append(r)
    with open(os.path.join(HERE, "verdicts.json"), "w") as fh:
        json.dump(uniq, fh, indent=0)
    seen, duniq = set(), []
    for r in dnf_rows:
        k = (r["model"], r["formula"])
        if k not in seen:
            seen.add(k)
            duniq.append(r)
    with open(os.path.join(HERE, "verdicts_dnf.json"), "w") as fh:
        json.dump(duniq, fh, indent=0)
    print(f"{len(uniq)} verdict rows and {len(duniq)} disjunctive rows over {sum(1 for n in nets.values() if n)} "
          f"models; skipped {len(skipped)}")
    for s in skipped:
        print("  skip", *s)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_fixtures.py <path of the reference checkout>")
    main(sys.argv[1])
