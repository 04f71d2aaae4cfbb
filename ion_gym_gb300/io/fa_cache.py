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
from pathlib import Path

import numpy as np

from ion_gym_gb300.io.publish import staged, write_json

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
    if _complete(dest):
        return key
    with staged(dest, folder=True, keep_if=_complete) as tmp:
        manifest = {}
        for name, a in arrays.items():
            a = np.ascontiguousarray(a)
            np.save(os.path.join(tmp, name + ".npy"), a)
            manifest[name] = {"shape": list(a.shape), "dtype": str(a.dtype),
                              "sha_head": sha_head(a)}
        meta = {"key": key, "version": CACHE_VERSION, "spec": spec,
                "arrays": manifest}
        # meta.json is the completeness marker: written last
        with open(os.path.join(tmp, "meta.json"), "w", encoding="utf-8") as f:
            json.dump(meta, f, indent=1)
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
                      verbose=False, precision=None):
    """physics/build_stl3d._solve_stl3d_bases (build_stl3d.py:835-849): the
    basis door at V_BASIS and STL3D_SOLVE_TOL, returned as float32 unit
    bases.  precision (not in the reference signature): None / "fp64" runs
    the reference's V-cycle (its bits), "mixed" the batched mixed-precision
    session to the same tolerance, its unit bases formed on the device
    (multigrid3d.solve_unit_bases_mg); solve_code.solve_code_key(precision)
    keys the cache entry on the choice."""
    from ion_gym_gb300.physics.multigrid3d import solve_unit_bases_mg
    # mirror_axes only shapes theta, which the STL route does not build
    # (theta None), as in the reference
    return solve_unit_bases_mg(masks, v_basis=V_BASIS, tol=STL3D_SOLVE_TOL,
                               stencil="ghost_linear", verbose=verbose,
                               precision=precision)


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


PROVENANCE = "provenance.json"


def _read_json(path):
    """(object, None) of a JSON file, (None, reason) when it is unreadable,
    (None, None) when it does not exist."""
    try:
        with open(path, encoding="utf-8") as f:
            return json.load(f), None
    except FileNotFoundError:
        return None, None
    except (OSError, ValueError) as e:
        return None, f"{type(e).__name__}: {e}"


def _records(entry_dir):
    """(provenance records, problem) of an entry: [] and a reason when the
    sidecar is unreadable or not a list of records."""
    recs, why = _read_json(os.path.join(entry_dir, PROVENANCE))
    if why is None and recs is not None and not isinstance(recs, list):
        why = f"expected a list of records, found {type(recs).__name__}"
    if why is not None or recs is None:
        return [], why
    return [r for r in recs if isinstance(r, dict)], None


def latest_spec_json(records):
    """The producing spec of the newest record that carries one, or None."""
    for r in reversed(records):
        if r.get("spec_json"):
            return r["spec_json"]
    return None


def annotate(spec_or_key, name, label=None, root=None, spec_json=None):
    """Record in the entry's provenance.json sidecar that the spec `name`
    (with `label`) produced or resolved it (fa_cache.py:219-272): one
    {name, label, when[, spec_json]} record per (name, label); naming the
    same pair again refreshes its time and spec_json.  The sidecar is
    descriptive only: an unreadable one is started afresh, and a failed
    write is reported on stdout, never raised.  Missing entries and empty
    names are ignored."""
    import time
    key = spec_or_key if isinstance(spec_or_key, str) else spec_key(spec_or_key)
    name = (name or "").strip()
    entry = os.path.join(os.path.expanduser(_root(root)), key)
    if not name or not os.path.isdir(entry):
        return
    recs, why = _records(entry)
    if why is not None:
        print(f"fa_cache: entry {key}: starting a new provenance record "
              f"list, the old one could not be read ({why})")
    stamp = {"when": time.strftime("%Y-%m-%d %H:%M")}
    if spec_json is not None:
        stamp["spec_json"] = spec_json
    mine = [r for r in recs if (r.get("name"), r.get("label")) == (name, label)]
    if mine:
        mine[0].update(stamp)
    else:
        recs.append({"name": name, "label": label, **stamp})
    try:
        write_json(os.path.join(entry, PROVENANCE), recs)
    except OSError as e:
        print(f"fa_cache: entry {key}: provenance not written ({e})")


def _describe(entry_dir):
    """One inventory row of an entry folder; never raises."""
    files = []
    for dp, _, fn in os.walk(entry_dir):
        files += [os.path.join(dp, f) for f in fn]
    size = unsized = 0
    for f in files:
        try:
            size += os.path.getsize(f)
        except OSError:
            unsized += 1
    row = {"key": os.path.basename(entry_dir), "bytes": size,
           "unsized_files": unsized,
           "arrays": sum(f.endswith(".npy") for f in files),
           "mtime": os.path.getmtime(entry_dir), "spec_name": None,
           "shape": None, "produced_by": [], "descriptor": None,
           "has_spec_json": False, "problems": []}
    recs, why = _records(entry_dir)
    if why is not None:
        row["problems"].append(f"{PROVENANCE} unreadable ({why})")
    row["produced_by"] = [r["name"] for r in recs if r.get("name")]
    labels = [r["label"] for r in recs if r.get("label")]
    row["descriptor"] = labels[-1] if labels else None
    row["has_spec_json"] = latest_spec_json(recs) is not None
    meta, why = _read_json(os.path.join(entry_dir, "meta.json"))
    if why is not None:
        row["problems"].append(f"meta.json unreadable ({why})")
    elif isinstance(meta, dict):
        spec = meta.get("spec")
        if isinstance(spec, dict):
            row["spec_name"] = spec.get("name")
        shapes = [a.get("shape") for a in (meta.get("arrays") or {}).values()
                  if isinstance(a, dict)]
        row["shape"] = shapes[0] if shapes else None
    return row


def entries(root=None):
    """Inventory of the cache (fa_cache.py:275-330): one row per entry
    folder, in key order -- key, bytes on disk (unsized_files counts files
    whose size could not be read), .npy count, mtime, the stored spec's
    name, the first array's shape, the names that produced it, its latest
    label, whether a producing spec JSON is recorded, and the problems met
    reading it."""
    root = os.path.expanduser(_root(root))
    if not os.path.isdir(root):
        return []
    return [_describe(os.path.join(root, n)) for n in sorted(os.listdir(root))
            if not n.startswith(".") and os.path.isdir(os.path.join(root, n))]
