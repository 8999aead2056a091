"""CPU checks that the bindings stay ABI-exact with include/mdsx.h: the ctypes
table (massivemds_gb300/_lib.py) gives every entry point the header's number of
parameters, and the binding snippets of INTEGRATION.md (the reference-side
factory patch, the ctypes, JNI, Rcpp and row-partition stubs a maintainer
would add) name only declared entry points and constants and call each entry
point with its declared number of arguments."""
import os
import re

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "mdsx.h")
INTEGRATION = os.path.join(REPO, "INTEGRATION.md")


def _strip_comments(text):
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    return re.sub(r"//[^\n]*", " ", text)


def _split_top_level(args):
    """Arguments of a call or parameter list, split at commas outside brackets."""
    parts, depth, cur = [], 0, []
    for ch in args:
        if ch in "([{":
            depth += 1
        elif ch in ")]}":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append("".join(cur).strip())
            cur = []
        else:
            cur.append(ch)
    last = "".join(cur).strip()
    if last or parts:
        parts.append(last)
    return parts


def _balanced(text, open_at):
    """The text between the parenthesis at open_at and its match, or None."""
    depth = 0
    for i in range(open_at, len(text)):
        if text[i] == "(":
            depth += 1
        elif text[i] == ")":
            depth -= 1
            if depth == 0:
                return text[open_at + 1:i]
    return None


def header_prototypes():
    """{name: parameter count} of every function include/mdsx.h declares."""
    text = _strip_comments(open(HEADER).read())
    protos = {}
    for m in re.finditer(r"\b(mdsx_[a-z0-9_]+)\s*\(", text):
        before = text[:m.start()].rstrip()
        # a declaration: the name follows a return type, not an operator or '('
        if not re.search(r"(\bint|\bdouble|\bvoid|\bconst char\s*\*|\blong)\s*\**$", before):
            continue
        params = _balanced(text, m.end() - 1)
        if params is None:
            continue
        parts = _split_top_level(params)
        protos[m.group(1)] = 0 if parts in ([], ["void"]) else len(parts)
    return protos


def snippet_blocks():
    text = open(INTEGRATION).read()
    return re.findall(r"```[a-z]*\n(.*?)```", text, flags=re.S)


def test_header_prototypes_parse():
    protos = header_prototypes()
    for name in ("mdsx_create", "mdsx_update_locations", "mdsx_get_sum_of_increments",
                 "mdsx_batch_create", "mdsx_sweep_f32_noalloc", "mdsx_hmc_run"):
        assert name in protos, name
    assert protos["mdsx_create"] == 5
    assert protos["mdsx_get_sum_of_increments"] == 2


def test_ctypes_table_matches_header_arity():
    from massivemds_gb300 import _lib

    protos = header_prototypes()
    assert set(_lib.SIGNATURES) == set(protos), set(_lib.SIGNATURES) ^ set(protos)
    for name, (_, args) in _lib.SIGNATURES.items():
        assert len(args) == protos[name], (name, len(args), protos[name])


def test_snippets_name_only_declared_symbols():
    declared = open(HEADER).read()
    for root, _, files in os.walk(os.path.join(REPO, "include")):
        for f in files:
            declared += open(os.path.join(root, f)).read()
    names = set()
    for block in snippet_blocks():
        names |= set(re.findall(r"\b(mdsx_[a-z0-9]+(?:_[a-z0-9]+)*|MDSX_[A-Z0-9_]+)\b", block))
    assert names, "no bindings found"
    missing = sorted(n for n in names if not re.search(r"\b" + re.escape(n) + r"\b", declared))
    assert not missing, missing


def test_snippet_calls_have_the_declared_arity():
    protos = header_prototypes()
    calls = 0
    for block in snippet_blocks():
        for m in re.finditer(r"\b(mdsx_[a-z0-9_]+)\s*\(", block):
            name = m.group(1)
            if name not in protos:
                continue
            args = _balanced(block, m.end() - 1)
            if args is None or "..." in args:  # an elided argument list in prose
                continue
            n = len(_split_top_level(args))
            assert n == protos[name], (name, args, protos[name])
            calls += 1
    assert calls >= 15, calls
