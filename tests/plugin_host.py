"""Test helper: builds the plugin test host (tests/plugin/host.cc) and runs
jobs through it (see host.cc for the binary job format).  Test
infrastructure only."""
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def build_host(out_dir):
    exe = os.path.join(out_dir, "plugin_host")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(REPO, "include"),
                    os.path.join(HERE, "plugin", "host.cc"), "-ldl", "-o", exe], check=True)
    return exe


def _i(*xs):
    return np.asarray(xs, dtype=np.int32).tobytes()


def job_frames(coord, atype, box, kind=0):
    coord = np.asarray(coord, np.float64).reshape(-1)
    atype = np.asarray(atype, np.int32).reshape(-1)
    na = atype.size if kind != 3 else None
    if kind == 3:  # mixed types: atype is [nframes, natoms]
        nf, na = np.asarray(atype).reshape(box.shape[0] if box is not None else 1, -1).shape
    else:
        nf = coord.size // (3 * na)
    b = b"" if box is None else np.asarray(box, np.float64).reshape(-1).tobytes()
    return _i(kind, nf, na) + coord.tobytes() + atype.tobytes() + _i(0 if box is None else 1) + b


def job_nlist(ext, ext_t, nghost, ilist, rows, ago=0):
    ext = np.asarray(ext, np.float64).reshape(-1)
    ext_t = np.asarray(ext_t, np.int32)
    nn = np.array([len(r) for r in rows], np.int32)
    flat = np.concatenate([np.asarray(r, np.int32) for r in rows]) if rows else np.zeros(0, np.int32)
    return (_i(2, ext_t.size, nghost) + ext.tobytes() + ext_t.tobytes() + _i(len(ilist)) +
            np.asarray(ilist, np.int32).tobytes() + nn.tobytes() + flat.tobytes() + _i(ago))


def run(exe, plugin, model, jobs, env=None):
    """-> (returncode, stdout, [(e, f, v, ae, av) per job])"""
    with tempfile.TemporaryDirectory() as d:
        jin, jout = os.path.join(d, "jobs.bin"), os.path.join(d, "out.bin")
        with open(jin, "wb") as f:
            f.write(_i(len(jobs)) + b"".join(jobs))
        r = subprocess.run([exe, plugin, model, jin, jout], capture_output=True, text=True, timeout=600,
                           env=dict(os.environ, **(env or {})))
        outs = []
        if os.path.exists(jout):
            buf = open(jout, "rb").read()
            p = 0
            while p < len(buf):
                arrs = []
                for _ in range(5):
                    n = int(np.frombuffer(buf, np.int64, 1, p)[0])
                    p += 8
                    arrs.append(np.frombuffer(buf, np.float64, n, p).copy())
                    p += 8 * n
                outs.append(tuple(arrs))
        return r.returncode, r.stdout + r.stderr, outs
