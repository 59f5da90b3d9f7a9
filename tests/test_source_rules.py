"""Source rules of the CUDA kernels that no compiler checks.

A warp collective (__shfl*_sync, __reduce_*_sync, __ballot_sync, __any_sync, __all_sync) with a
full mask must be executed by every lane of the warp.  One placed in the arm of a conditional
expression (`cond ? a : __shfl_sync(...)`) or after a short-circuit operator is skipped by the
lanes that take the other arm: the lanes that execute it then wait for lanes that never
arrive.  Such collectives are computed unconditionally and selected afterwards."""
import os
import re

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "radialbasisfunctions.jl_gb300",
                    "csrc")
COLLECTIVE = r"__(shfl(_up|_down|_xor)?|reduce_\w+|ballot|any|all)_sync\s*\("


def statements():
    for name in sorted(os.listdir(CSRC)):
        if not name.endswith((".cu", ".cuh")):
            continue
        text = open(os.path.join(CSRC, name)).read()
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"[^;{}]*;", text):
            yield name, text.count("\n", 0, m.start()) + 1, m.group(0)


def test_no_warp_collective_in_a_conditional_arm():
    bad = []
    for name, line, st in statements():
        c = re.search(COLLECTIVE, st)
        if not c:
            continue
        head = st[:c.start()]
        # a '?' or a short-circuit operator before the collective in the same statement
        if re.search(r"\?|&&|\|\|", head.replace("?:", "")):
            bad.append(f"{name}:{line}: {st.strip()[:120]}")
    assert not bad, "warp collectives that some lanes may skip:\n" + "\n".join(bad)
