"""The host emitter-tree build of the product (sl_emitter_tree: buildEmitterTree + packEmitNodes, src/lighting.js:99-169)
against the oracle's restatement, node for node, with its skip links checked against the cut walk they replace (a
48-entry stack popping hi first) and its derivative table checked against central differences of the oracle's
float64 build.  Host only: no device is touched."""
import ctypes as C

import numpy as np
import pytest

from splatlight_gb300 import scene
from splatlight_gb300.structs import GAUSSIAN

NONE = 0xFFFFFFFF


@pytest.fixture(scope="module")
def native():
    from splatlight_gb300 import build
    build.build()
    from splatlight_gb300 import _native
    return _native


def _tree(native, rec, scale=None, dtab=False):
    n = len(rec)
    r = np.ascontiguousarray(rec, dtype=GAUSSIAN)
    nodes = np.zeros((2 * n - 1, 24), np.float32)
    tab = np.zeros((2 * n - 1, n, 9), np.float32) if dtab else None
    sc = None if scale is None else np.ascontiguousarray(scale, np.float64)
    root = C.c_uint32()
    native.check(native.lib().sl_emitter_tree(r.ctypes.data, n, None if sc is None else sc.ctypes.data,
                                              nodes.ctypes.data, None if tab is None else tab.ctypes.data,
                                              C.byref(root)))
    return nodes, root.value, tab


def _emitter_sets():
    yield "cornell 8", scene.cornell(4096).emitters
    yield "hill 32", scene.hill(4096, seed=1).emitters
    e = scene.hill(4096, seed=2).emitters[:5].copy()
    e["mu"][3] = e["mu"][1]                              # a tie on every axis: the stable split keeps index order
    yield "ties 5", e
    yield "one", e[:1]


def _stack_cut(nodes, root, P, theta=4.0):
    """The cut as a 48-entry stack walks it (hi popped first; a full stack neither uses nor refines a node)."""
    u = nodes.view(np.uint32)
    out, st = [], [root]
    while st:
        k = st.pop()
        lo, hi = u[k, 11], u[k, 15]
        if lo == NONE:
            out.append(k)
            continue
        d = P - nodes[k, :3].astype(np.float64)
        if d @ d > theta * theta * float(nodes[k, 3]) ** 2:
            out.append(k)
        elif len(st) + 2 <= 48:
            st += [lo, hi]
    return out


def _skip_cut(nodes, root, P, theta=4.0):
    """The shading pass's stackless walk over the skip links (word 7) and full-stack marks (word 19)."""
    u = nodes.view(np.uint32)
    out, k, guard = [], root, 0
    while k != NONE and guard < 1 << 16:
        assert k < len(nodes)
        lo, hi, skip = u[k, 11], u[k, 15], u[k, 7]
        d = P - nodes[k, :3].astype(np.float64)
        use = lo == NONE or d @ d > theta * theta * float(nodes[k, 3]) ** 2
        if use:
            out.append(k)
            k = skip
        else:
            k = hi if u[k, 19] == 0 else skip
        guard += 1
    return out


@pytest.mark.parametrize("name,rec", list(_emitter_sets()), ids=lambda x: x if isinstance(x, str) else "")
def test_tree_node_for_node(native, orc, name, rec):
    nodes, root, _ = _tree(native, rec)
    ref, ref_root, _ = orc.emitter_tree(np.ascontiguousarray(rec, GAUSSIAN).view(np.float32))
    assert root == ref_root
    words = [w for w in range(24) if w not in (7, 19)]   # 7 and 19: the skip links, which the restatement lacks
    assert nodes[:, words].tobytes() == ref[:, words].tobytes()
    rng = np.random.default_rng(0)
    lo, hi = rec["mu"].min(axis=0) - 3.0, rec["mu"].max(axis=0) + 3.0
    for P in rng.uniform(lo, hi, (300, 3)):
        assert _skip_cut(nodes, root, P) == _stack_cut(nodes, root, P)


def test_derivative_table(native, orc):
    rec = scene.hill(4096, seed=1).emitters[:8]
    scale = np.linspace(0.7, 1.4, 8)
    nodes, root, tab = _tree(native, rec, scale, dtab=True)
    ref, ref_root = orc.emitter_tree_d(np.ascontiguousarray(rec, GAUSSIAN).view(np.float32), scale)
    assert root == ref_root
    assert np.allclose(nodes[:, 12:15], ref[:, 10:13], rtol=1e-6)
    for k in range(8):
        h = 1e-4 * scale[k]
        sp, sm = scale.copy(), scale.copy()
        sp[k] += h
        sm[k] -= h
        tp, _ = orc.emitter_tree_d(np.ascontiguousarray(rec, GAUSSIAN).view(np.float32), sp)
        tm, _ = orc.emitter_tree_d(np.ascontiguousarray(rec, GAUSSIAN).view(np.float32), sm)
        fd = (tp - tm) / (2 * h)
        want = np.concatenate([fd[:, 10:13], fd[:, 4:10]], axis=1)          # Le rgb, M xx yy zz xy xz yz
        got = tab[:, k, :].astype(np.float64)
        err = np.abs(got - want).max() / max(np.abs(want).max(), 1e-30)
        assert err < 1e-4, (k, err)
        # an emitter's intensity moves its own leaf's Le and no other leaf's
        leaves = nodes.view(np.uint32)[:, 11] == NONE
        own = leaves & (nodes.view(np.uint32)[:, 15] == k)
        assert np.all(tab[leaves & ~own, k, :3] == 0.0) and np.any(tab[own, k, :3] != 0.0)
