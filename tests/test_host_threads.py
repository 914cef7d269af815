"""The host setup passes (nested dissection, the permuted patterns, the
symbolic row structure) give the same result on any number of host threads.

The row fill runs disjoint subtrees of a supernodal tree predicted from the
elimination tree on several threads and falls back to the serial recursion if
any prediction is wrong; the dissection runs its top levels' halves
concurrently; the per-column sorts are split into column ranges.  Each case is
ordered and analysed in a child process with RSCHOL_HOST_THREADS set to 1, 3
and 8, and the permutation, the supernode partition and every supernode's row
list must be identical.  The cases are large enough (n >= 4096, >= 64
supernodes) for every parallel pass to engage.
"""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

DIGEST = r"""
import sys, json, hashlib; sys.path.insert(0, %r)
import numpy as np
import rank_structured_cholesky_gb300 as rs
from oracle import pyoracle as po
out = {}
cases = [("3d24", rs.diffusion(3, 24, sigma=1.0, seed=1), True, {}),
         ("3d20 graph", rs.diffusion(3, 20, sigma=1.0, seed=1), False, {}),
         ("2d96 compressing", rs.diffusion(2, 96, sigma=1.0, seed=1), True, dict(max_dense_block=16, max_diag_block=32)),
         ("el12 graph", rs.elasticity(12), False, {})]
for name, p, use_xyz, prm in cases:
    F = po.OracleFactor(p.colptr, p.rowind, p.vals, p.xyz if use_xyz else None, prm)
    h = hashlib.sha256(F.perm().tobytes())
    nn = F.num_nodes()
    for j in range(nn):
        i = F.node_info(j)
        h.update(np.array([i["c0"], i["c1"], i["compressed"], i["m"], i["n_stored"], i["interior"]],
                          dtype=np.int64).tobytes())
        h.update(F.node_rows(j).tobytes())
    out[name] = [p.n, nn, h.hexdigest()]
print(json.dumps(out))
""" % ROOT


def digests(threads):
    env = dict(os.environ)
    env["RSCHOL_HOST_THREADS"] = str(threads)
    r = subprocess.run([sys.executable, "-c", DIGEST], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_setup_passes_independent_of_thread_count():
    one = digests(1)
    for name, (n, nn, _) in one.items():
        assert n >= 4096 and nn >= 64, (name, n, nn)
    for t in (3, 8):
        assert digests(t) == one, t


PARALLEL_CHECK = r"""
#include <atomic>
#include <cstdio>
#include <stdexcept>
#include <vector>
#include "parallel.h"
int main() {
  using namespace rschol;
  const long long n = 100003;
  std::vector<int> hits(n, 0);
  parallel_chunks(n, 1000, [&](long long b, long long e) {
    for (long long i = b; i < e; ++i) hits[i]++;
  });
  for (long long i = 0; i < n; ++i)
    if (hits[i] != 1) return 1;
  std::atomic<int> calls(0), mask(0);
  run_workers(5, [&](int t) { calls++; mask |= 1 << t; });
  if (calls != 5 || mask != 31) return 2;
  bool caught = false;
  try {
    parallel_chunks(n, 10, [&](long long b, long long e) {
      if (b <= 77777 && 77777 < e) throw std::runtime_error("chunk failed");
    });
  } catch (const std::runtime_error&) {
    caught = true;
  }
  if (!caught) return 3;
  std::printf("%d\n", host_threads());
  return 0;
}
"""


def test_parallel_helpers(tmp_path):
    """Every index visited once, every worker run once, a worker's exception
    rethrown on the calling thread; RSCHOL_HOST_THREADS is honoured."""
    src = tmp_path / "par.cpp"
    src.write_text(PARALLEL_CHECK)
    exe = tmp_path / "par"
    host = os.path.join(ROOT, "rank_structured_cholesky_gb300", "csrc", "host")
    subprocess.run(["g++", "-std=c++17", "-O2", "-pthread", "-I", host, str(src), "-o", str(exe)], check=True,
                   stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    for threads in ("1", "4", "16"):
        env = dict(os.environ, RSCHOL_HOST_THREADS=threads)
        r = subprocess.run([str(exe)], env=env, capture_output=True, text=True, timeout=60)
        assert r.returncode == 0, (threads, r.returncode)
        assert r.stdout.strip() == threads
