"""Static check of the Python sources (no GPU): every name a function reads from module scope
is defined there, imported, or a builtin -- the error a workload branch of bench.py that the
CPU tests do not execute would otherwise only show on the GPU machine."""
import builtins
import glob
import os
import symtable

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def undefined_globals(path):
    src = open(path).read()
    top = symtable.symtable(src, path, "exec")
    defined = {s.get_name() for s in top.get_symbols() if s.is_assigned() or s.is_imported()}
    defined |= {c.get_name() for c in top.get_children()}
    bad = []

    def walk(t):
        for s in t.get_symbols():
            n = s.get_name()
            if s.is_global() and s.is_referenced() and not s.is_assigned() and n not in defined \
                    and not hasattr(builtins, n) and n not in ("__file__", "__name__"):
                bad.append((t.get_name(), n))
        for c in t.get_children():
            walk(c)

    walk(top)
    return bad


def test_no_undefined_module_names():
    paths = [os.path.join(ROOT, "bench.py"), os.path.join(ROOT, "__graft_entry__.py")]
    paths += sorted(glob.glob(os.path.join(ROOT, "cgenie_gb300", "*.py")))
    paths += sorted(glob.glob(os.path.join(ROOT, "oracle", "*.py")))
    problems = {os.path.relpath(p, ROOT): undefined_globals(p) for p in paths}
    problems = {k: v for k, v in problems.items() if v}
    assert not problems, problems


def test_ensemble_add_many_of_nothing_calls_nothing():
    """Ensemble.add_many([]) returns [] without a library call (no GPU needed)."""
    from cgenie_gb300.ensemble import Ensemble
    e = object.__new__(Ensemble)
    e.members, e.tile, e.table, e._current_tile, e.use_graph = {}, (0, 0), {}, None, False
    assert e.add_many([]) == []
