"""The solved-basis cache on disk, in the reference's layout
(ion_gym io/fa_cache.py:106-201, entries written by
physics/build_stl3d.py:919-924), so caches written here are read by the
reference and the other way round.

    <ION_GYM_CACHE or ~/.ion_gym_cache>/<key>/
        meta.json         {"key", "version": 2, "spec", "arrays": {name:
                           {"shape", "dtype", "sha_head"}}}
        basis_<i>.npy     float32 unit basis of electrode i, (nx, ny, nz)
        labels.npy        uint8 electrode index per node, 0 = vacuum

key = the first 16 hex digits of sha256 over the canonical JSON of
{"v": CACHE_VERSION, "spec": spec} (sorted keys, compact separators, floats
rounded to 10 digits); sha_head = the first 16 hex digits of sha256 over the
first 4096 bytes of the array.  Entries are published atomically: the arrays
and meta.json are written to a temporary directory that is renamed into
place; the first writer wins and a loser's copy is removed.
"""
import hashlib
import json
import os
import shutil
import tempfile
from pathlib import Path

import numpy as np

CACHE_VERSION = 2


def cache_root():
    """ION_GYM_CACHE if set, else ~/.ion_gym_cache, resolved at call time
    (io/paths.py:251-259)."""
    env = os.environ.get("ION_GYM_CACHE")
    return Path(env).expanduser() if env else Path.home() / ".ion_gym_cache"


def _root(root):
    return str(cache_root()) if root is None else str(root)


def _canonical(obj):
    def norm(x):
        if isinstance(x, bool) or x is None or isinstance(x, str):
            return x
        if isinstance(x, (float, np.floating)):
            return round(float(x), 10)
        if isinstance(x, (np.integer,)):
            return int(x)
        if isinstance(x, np.ndarray):
            return [norm(v) for v in x.tolist()]
        if isinstance(x, (list, tuple)):
            return [norm(v) for v in x]
        if isinstance(x, dict):
            return {k: norm(x[k]) for k in sorted(x)}
        return x
    return json.dumps(norm(obj), sort_keys=True, separators=(",", ":"))


def spec_key(spec):
    """16-hex key of a JSON-able spec (fa_cache.py:82-86)."""
    payload = _canonical({"v": CACHE_VERSION, "spec": spec})
    return hashlib.sha256(payload.encode()).hexdigest()[:16]


def sha_head(a, n=4096):
    raw = np.ascontiguousarray(a).view(np.uint8).reshape(-1)[:n].tobytes()
    return hashlib.sha256(raw).hexdigest()[:16]


def _complete(dest):
    try:
        with open(os.path.join(dest, "meta.json"), encoding="utf-8") as f:
            names = list(json.load(f).get("arrays") or {})
    except (OSError, ValueError, AttributeError):
        return False
    return all(os.path.exists(os.path.join(dest, n + ".npy")) for n in names)


def store(spec, arrays, root=None):
    """Write {name: array} under the spec's key atomically; returns the key.
    A complete entry that already exists is kept; an incomplete one is
    replaced."""
    root = _root(root)
    key = spec_key(spec)
    dest = os.path.join(root, key)
    if os.path.exists(os.path.join(dest, "meta.json")):
        if _complete(dest):
            return key
        shutil.rmtree(dest, ignore_errors=True)
    os.makedirs(root, exist_ok=True)
    tmp = tempfile.mkdtemp(prefix=f".{key}.", dir=root)
    published = False
    try:
        manifest = {}
        for name, a in arrays.items():
            a = np.ascontiguousarray(a)
            np.save(os.path.join(tmp, name + ".npy"), a)
            manifest[name] = {"shape": list(a.shape), "dtype": str(a.dtype),
                              "sha_head": sha_head(a)}
        meta = {"key": key, "version": CACHE_VERSION, "spec": spec,
                "arrays": manifest}
        with open(os.path.join(tmp, "meta.json"), "w", encoding="utf-8") as f:
            json.dump(meta, f, indent=1)
            f.flush()
            os.fsync(f.fileno())
        try:
            os.replace(tmp, dest)
            published = True
        except OSError:
            if not os.path.exists(os.path.join(dest, "meta.json")):
                raise
    finally:
        if not published and os.path.isdir(tmp):
            shutil.rmtree(tmp, ignore_errors=True)
    return key


def load(spec_or_key, root=None, mmap=True, names=None):
    """(arrays, meta) of an entry, (None, None) on a miss; raises IOError on
    a truncated or tampered entry (shape, dtype or head hash mismatch)."""
    root = _root(root)
    key = (spec_or_key if isinstance(spec_or_key, str)
           and len(spec_or_key) == 16 else spec_key(spec_or_key))
    dest = os.path.join(root, key)
    mpath = os.path.join(dest, "meta.json")
    if not os.path.exists(mpath):
        return None, None
    with open(mpath, encoding="utf-8") as f:
        meta = json.load(f)
    if meta.get("key") != key or meta.get("version") != CACHE_VERSION:
        return None, None
    out = {}
    for name in (names or list(meta["arrays"])):
        p = os.path.join(dest, name + ".npy")
        if not os.path.exists(p):
            raise IOError(f"cache {key}: missing array {name}")
        try:
            a = np.load(p, mmap_mode="r" if mmap else None)
        except (ValueError, OSError, EOFError) as e:
            raise IOError(f"cache {key}: {name} unreadable ({e}): truncated "
                          f"or corrupt entry")
        m = meta["arrays"][name]
        if list(a.shape) != m["shape"] or str(a.dtype) != m["dtype"]:
            raise IOError(f"cache {key}: {name} shape/dtype mismatch: "
                          f"truncated or corrupt entry")
        if m.get("sha_head") is None or sha_head(a) != m["sha_head"]:
            raise IOError(f"cache {key}: {name} head hash mismatch: corrupt "
                          f"entry")
        out[name] = a
    return out, meta


def verify(spec_or_key, root=None):
    try:
        arrs, _ = load(spec_or_key, root=root, mmap=False)
    except (IOError, OSError):
        return False
    return arrs is not None


# ------------------------------------------------------------ basis entries
V_BASIS = 1e4          # the basis excitation (physics/build_planar.py:106)
STL3D_SOLVE_TOL = 1e-4  # physics/build_stl3d.py:40


def solve_stl3d_bases(masks, mirror_axes=(False, False, False),
                      verbose=False):
    """physics/build_stl3d._solve_stl3d_bases (build_stl3d.py:835-849): the
    V-cycle basis door at V_BASIS and STL3D_SOLVE_TOL, returned as float32
    unit bases."""
    from ion_gym_gb300.physics.multigrid3d import solve_bases_mg
    bases = solve_bases_mg(masks, mirror=mirror_axes, v_basis=V_BASIS,
                           tol=STL3D_SOLVE_TOL, stencil="ghost_linear",
                           verbose=verbose)
    return {i: (b / V_BASIS).astype(np.float32) for i, b in bases.items()}


def store_bases(spec, bases, masks, root=None):
    """Write a basis set as build_stl3d does (build_stl3d.py:919-924):
    basis_<i> float32 and labels uint8 (the electrode index per node, later
    masks win where they overlap)."""
    shape = np.asarray(next(iter(masks.values()))).shape
    lab = np.zeros(shape, np.uint8)
    for i, m in masks.items():
        lab[np.asarray(m, bool)] = i
    arrays = {f"basis_{i}": np.asarray(b, np.float32) for i, b in bases.items()}
    arrays["labels"] = lab
    return store(spec, arrays, root=root)


def load_bases(spec_or_key, root=None):
    """({i: basis}, {i: mask}) of a cached basis set, or (None, None)."""
    arrs, _ = load(spec_or_key, root=root)
    if arrs is None:
        return None, None
    bases = {int(k.split("_")[1]): v for k, v in arrs.items()
             if k.startswith("basis_")}
    lab = arrs["labels"]
    return bases, {i: (lab == i) for i in bases}


def annotate(spec_or_key, name, label=None, root=None, spec_json=None):
    """Record which named spec produced or resolved an entry in its
    provenance.json sidecar (fa_cache.py:219-272): a list of {name, label,
    when[, spec_json]} records; a repeated (name, label) refreshes its time
    (and spec_json).  Descriptive only: an unreadable sidecar is rebuilt
    and a write failure is reported, never raised."""
    import time
    key = (spec_or_key if isinstance(spec_or_key, str) else spec_key(spec_or_key))
    name = (name or "").strip()
    if not name:
        return
    dest = os.path.join(os.path.expanduser(_root(root)), key)
    if not os.path.isdir(dest):
        return
    ppath = os.path.join(dest, "provenance.json")
    recs = []
    if os.path.exists(ppath):
        try:
            with open(ppath, encoding="utf-8") as f:
                recs = json.load(f)
            if not isinstance(recs, list):
                raise ValueError(f"expected a list, got {type(recs).__name__}")
        except (OSError, ValueError) as e:
            print(f"fa_cache: provenance sidecar unreadable for {key} "
                  f"({e}) — rebuilding it (descriptive data only).")
            recs = []
    now = time.strftime("%Y-%m-%d %H:%M")
    for r in recs:
        if r.get("name") == name and r.get("label") == label:
            r["when"] = now
            if spec_json is not None:
                r["spec_json"] = spec_json
            break
    else:
        rec = dict(name=name, label=label, when=now)
        if spec_json is not None:
            rec["spec_json"] = spec_json
        recs.append(rec)
    try:
        fd, tmp = tempfile.mkstemp(dir=dest, prefix=".prov.")
        with os.fdopen(fd, "w") as f:
            json.dump(recs, f, indent=1)
        os.replace(tmp, ppath)
    except OSError as e:
        print(f"fa_cache: could not write provenance for {key} ({e})")


def entries(root=None):
    """[{key, arrays, spec_name, shape, produced_by, has_spec_json}] of the
    complete-or-not entries under root (fa_cache.py:275-330, the fields a
    field export needs)."""
    root = os.path.expanduser(_root(root))
    out = []
    if not os.path.isdir(root):
        return out
    for name in sorted(os.listdir(root)):
        p = os.path.join(root, name)
        if not os.path.isdir(p) or name.startswith("."):
            continue
        rec = dict(key=name, arrays=sum(f.endswith(".npy") for f in os.listdir(p)),
                   spec_name=None, shape=None, produced_by=[], has_spec_json=False,
                   problems=[])
        ppath = os.path.join(p, "provenance.json")
        if os.path.exists(ppath):
            try:
                with open(ppath, encoding="utf-8") as f:
                    precs = json.load(f)
                if isinstance(precs, list):
                    rec["produced_by"] = [r.get("name") for r in precs
                                          if isinstance(r, dict) and r.get("name")]
                    rec["has_spec_json"] = any(isinstance(r, dict) and r.get("spec_json")
                                               for r in precs)
            except (OSError, ValueError) as e:
                rec["problems"].append(
                    f"provenance.json unreadable ({type(e).__name__}: {e})")
        mp = os.path.join(p, "meta.json")
        if os.path.exists(mp):
            try:
                with open(mp, encoding="utf-8") as f:
                    meta = json.load(f)
                spec = meta.get("spec", {}) or {}
                rec["spec_name"] = spec.get("name") if isinstance(spec, dict) else None
                arrs = meta.get("arrays", {}) or {}
                if arrs:
                    rec["shape"] = next(iter(arrs.values())).get("shape")
            except (OSError, ValueError, KeyError, AttributeError) as e:
                rec["problems"].append(f"meta.json unreadable ({type(e).__name__}: {e})")
        out.append(rec)
    return out
