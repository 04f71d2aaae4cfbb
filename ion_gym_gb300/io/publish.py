"""Crash-safe publication of cache entries, bundles and sidecar files.

Every file or folder this package writes for other processes to read goes
through one mechanism: the content is written under a hidden temporary name
in the destination's own folder (so the final rename never crosses a file
system), flushed to disk, and then renamed onto the destination name.  A
reader therefore sees either the previous file, or the complete new one,
never a half-written one; a writer that fails leaves nothing behind.

    with staged(path) as tmp:            # a file
        np.savez_compressed(tmp, **members)
    with staged(folder, folder=True) as tmp:   # a folder
        ...write files into tmp...

A staged folder is published only when the destination does not hold a
complete entry already (`keep_if`): a concurrent writer that got there first
wins, and the late copy is dropped.
"""
import contextlib
import json
import os
import shutil
import tempfile


def _sync(path):
    """Flush a file (or a folder's entries) to stable storage."""
    flags = os.O_RDONLY | getattr(os, "O_DIRECTORY", 0) * os.path.isdir(path)
    try:
        fd = os.open(path, flags)
    except OSError:
        return
    try:
        os.fsync(fd)
    except OSError:
        pass
    finally:
        os.close(fd)


def _discard(path):
    if os.path.isdir(path):
        shutil.rmtree(path, ignore_errors=True)
    elif os.path.exists(path):
        os.remove(path)


@contextlib.contextmanager
def staged(dest, folder=False, keep_if=None):
    """Yield a temporary path beside `dest`; when the block ends normally,
    sync it and rename it onto `dest`.

    folder: stage a directory instead of a file.  keep_if(dest) -> bool,
    for folders: when it holds at publication time, the existing `dest`
    stays and the staged copy is dropped; otherwise an existing `dest` is
    removed and replaced.  The context value is the temporary path; on any
    exception it is removed and the exception propagates."""
    dest = os.fspath(dest)
    parent = os.path.dirname(os.path.abspath(dest)) or "."
    os.makedirs(parent, exist_ok=True)
    tag = "." + os.path.basename(dest) + "."
    if folder:
        tmp = tempfile.mkdtemp(prefix=tag, dir=parent)
    else:
        fd, tmp = tempfile.mkstemp(prefix=tag, suffix=".part", dir=parent)
        os.close(fd)
    try:
        yield tmp
        if folder:
            for name in os.listdir(tmp):
                _sync(os.path.join(tmp, name))
            if keep_if is not None and keep_if(dest):
                return
            if os.path.isdir(dest):
                shutil.rmtree(dest)
        _sync(tmp)
        try:
            os.replace(tmp, dest)
        except OSError:
            # a folder published by another writer in between wins
            if not (folder and keep_if is not None and keep_if(dest)):
                raise
    finally:
        _discard(tmp)


def write_bytes(dest, data):
    with staged(dest) as tmp:
        with open(tmp, "wb") as f:
            f.write(data)


def write_text(dest, text):
    write_bytes(dest, text.encode("utf-8"))


def write_json(dest, obj, indent=1, **kw):
    write_text(dest, json.dumps(obj, indent=indent, **kw))


def write_npz(dest, members):
    """A compressed .npz of {member: array}."""
    import numpy as np
    with staged(dest) as tmp:
        with open(tmp, "wb") as f:
            np.savez_compressed(f, **members)
