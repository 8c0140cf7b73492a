"""Runs the known-answer cases (known_answers.py) through the oracle in the
as-shipped FP32 precision of the reference and writes their metrics to
known_answers.json, which the GPU tests compare against (the oracle itself is
pinned bit for bit to the reference's FP32 run by the golden fixtures).

    python tests/golden/make_known_answers.py            # all cases (~25 min on 8 cores)
    python tests/golden/make_known_answers.py reflection convergence
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [HERE, os.path.dirname(os.path.dirname(HERE))]

import numpy as np  # noqa: E402

import known_answers as K  # noqa: E402
import oracle.asm_oracle as O  # noqa: E402

OUT = os.path.join(HERE, "known_answers.json")


def solve(u0, kw):
    p = O.OracleParams(**kw)
    return O.solve(u0, p, "fp32")


def reflection():
    return {n: K.reflection_ratio(solve(*K.reflection_case(n))[3]) for n in K.REFLECTION_CONFIGS}


def convergence():
    out = {}
    for name in K.CONV_CONFIGS:
        traces = []
        for s in K.CONV_STEPS:
            u0, kw = K.convergence_case(name, s)
            f = solve(u0, kw)[0]
            traces.append(np.asarray(f[f.shape[0] // 2, f.shape[1] // 2], np.float64))
        errs = K.pair_errors(traces)
        out[name] = {"pair_errors": errs, "rate": K.pair_rate(errs)}
    return out


def baffled():
    u0, kw, g = K.baffled_case()
    r = solve(u0, kw)
    on, lat = K.baffled_metrics(r[6], r[3], r[5], g)
    return {"onaxis_rms": on, "lateral_rms": lat}


def focused():
    u0, kw, g = K.focused_case()
    r = solve(u0, kw)
    on, lat, fe = K.focused_metrics(r[6], r[3], r[5], g)
    return {"onaxis_rms": on, "lateral_rms": lat, "focal_amp_err": fe}


CASES = {"reflection": reflection, "convergence": convergence, "baffled": baffled,
         "focused": focused}


def main(names):
    O.set_fft_backend("scipy", os.cpu_count())
    data = {}
    if os.path.exists(OUT):
        with open(OUT) as f:
            data = json.load(f)
    for n in names:
        t0 = time.time()
        data[n] = CASES[n]()
        print(n, data[n], f"{time.time() - t0:.0f} s", flush=True)
        with open(OUT, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main(sys.argv[1:] or list(CASES))
