"""Regenerate the golden fixtures in tests/golden/.

  ising2d_8x8_logdos.json -- the exact log density of states of the 8x8 periodic
      Ising model (Beale 1996) that MonteCarloX.jl ships as
      SpinSystems/data/exact_solutions/ising2D_8x8.csv and loads in
      SpinSystems/src/ising2d_exact.jl.  Read from the reference checkout.
  philox_kat.json -- Philox4x32-10 known-answer vectors (the published Random123
      kat_vectors inputs), recomputed with an independent implementation (PyTorch's
      at::Philox4_32 header, compiled with g++) when it is available.
  oracle_traj.json -- short checkerboard trajectories of the oracle, so that later
      edits of the oracle cannot drift silently.

Usage: python tests/golden/make_golden.py [path-to-MonteCarloX.jl checkout]
"""
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

KAT_INPUTS = [
    ([0x00000000, 0x00000000, 0x00000000, 0x00000000], [0x00000000, 0x00000000]),
    ([0xffffffff, 0xffffffff, 0xffffffff, 0xffffffff], [0xffffffff, 0xffffffff]),
    ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0]),
]


def dos(ref_root):
    path = os.path.join(ref_root, "SpinSystems", "data", "exact_solutions", "ising2D_8x8.csv")
    rows = []
    with open(path) as f:
        next(f)
        for line in f:
            e, v = line.strip().split(",")
            rows.append([int(e), float(v)])
    with open(os.path.join(HERE, "ising2d_8x8_logdos.json"), "w") as f:
        json.dump({"source": "SpinSystems/data/exact_solutions/ising2D_8x8.csv (Beale 1996)",
                   "L": 8, "energy_logdos": rows}, f, indent=0)


def kat():
    import torch
    inc = os.path.join(os.path.dirname(torch.__file__), "include")
    src = r'''
#include <ATen/core/PhiloxRNGEngine.h>
#include <cstdio>
int main(int argc, char** argv) {
  unsigned c[4], k[2];
  while (scanf("%x %x %x %x %x %x", &c[0], &c[1], &c[2], &c[3], &k[0], &k[1]) == 6) {
    at::Philox4_32 e((uint64_t)k[0] | ((uint64_t)k[1] << 32), (uint64_t)c[2] | ((uint64_t)c[3] << 32),
                     (uint64_t)c[0] | ((uint64_t)c[1] << 32));
    unsigned o0 = e(), o1 = e(), o2 = e(), o3 = e();
    printf("%08x %08x %08x %08x\n", o0, o1, o2, o3);
  }
}
'''
    with tempfile.TemporaryDirectory() as d:
        cpp, exe = os.path.join(d, "k.cpp"), os.path.join(d, "k")
        open(cpp, "w").write(src)
        subprocess.run(["g++", "-std=c++17", "-I" + inc, "-o", exe, cpp], check=True)
        inp = "".join("%x %x %x %x %x %x\n" % (*c, *k) for c, k in KAT_INPUTS)
        out = subprocess.run([exe], input=inp, capture_output=True, text=True, check=True).stdout.split("\n")
    vec = []
    for (c, k), line in zip(KAT_INPUTS, out):
        vec.append({"ctr": c, "key": k, "out": [int(x, 16) for x in line.split()]})
    with open(os.path.join(HERE, "philox_kat.json"), "w") as f:
        json.dump({"generator": "Philox4x32-10", "vectors": vec}, f, indent=1)


def traj():
    import numpy as np
    import oracle as O
    cases = []
    for model, L, alg, beta, D, h in [
        (O.ISING, [8, 8], O.METROPOLIS, 0.4407, 0.0, 0.0),
        (O.ISING, [8, 8], O.GLAUBER, 0.3, 0.0, 0.0),
        (O.ISING, [8, 8], O.HEATBATH, 0.6, 0.0, 0.25),
        (O.ISING, [4, 4, 6], O.METROPOLIS, 0.22, 0.0, 0.0),
        (O.BC, [8, 8], O.METROPOLIS, 0.5, 1.0, 0.0),
        (O.BC, [8, 8], O.HEATBATH, 0.7, 0.5, 0.1),
    ]:
        s = O.init_random(model, L, 42, 3)
        obs, att, acc = O.cb_sweep(s, model, L, alg, beta, 42, stream=3, nsweeps=12, D=D, h=h)
        cases.append({"model": model, "L": L, "alg": alg, "beta": beta, "D": D, "h": h, "seed": 42,
                      "stream": 3, "nsweeps": 12, "obs": obs.tolist(), "attempts": att, "accepted": acc,
                      "spins": s.astype(int).tolist()})
    with open(os.path.join(HERE, "oracle_traj.json"), "w") as f:
        json.dump(cases, f)


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MCX_REFERENCE_ROOT")
    if not ref:
        sys.exit("usage: make_golden.py <MonteCarloX.jl checkout>  (or set MCX_REFERENCE_ROOT)")
    dos(ref)
    kat()
    traj()
    print("golden fixtures written to", HERE)
