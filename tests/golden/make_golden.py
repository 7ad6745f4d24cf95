"""Extract the known-answer values of openPSTD's kernel unit tests into JSON.

Reads the reference's Boost.Test sources (test/Kernel/kernel_functions.cpp,
test/Kernel/WisdomCache.cpp, test/Kernel/Domain.cpp, test/Kernel/Scene.cpp)
and writes tests/golden/reference_kats.json with the literal expected values
those tests check.  Run it where the reference tree is present:

    python tests/golden/make_golden.py /path/to/openPSTD

The JSON is committed; the tests read only the JSON.
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _floats(text):
    return [float(x) for x in re.findall(r"[-+]?\d*\.?\d+(?:[eE][-+]?\d+)?", text)]


def _stream(src, name):
    """Values of `name << a, b, c;` (Eigen comma initialiser) in src."""
    m = re.search(re.escape(name) + r"\s*<<\s*([^;]*);", src)
    if not m:
        raise ValueError(f"{name} not found")
    return _floats(m.group(1))


def main(ref):
    kf = open(os.path.join(ref, "test/Kernel/kernel_functions.cpp")).read()
    wc = open(os.path.join(ref, "test/Kernel/WisdomCache.cpp")).read()
    dm = open(os.path.join(ref, "test/Kernel/Domain.cpp")).read()
    sc = open(os.path.join(ref, "test/Kernel/Scene.cpp")).read()
    out = {"source": "openPSTD test/Kernel/*.cpp known-answer values"}

    # test/Kernel/kernel_functions.cpp
    n2p = re.findall(r"BOOST_CHECK_EQUAL\(next_2_power\(([^)]*)\),\s*(\d+)\)", kf)
    out["next_2_power"] = [[float(a), int(b)] for a, b in n2p]
    one = kf[kf.index("test_rho_array_one_neighbour"):kf.index("test_rho_array_two_neighbour")]
    two = kf[kf.index("test_rho_array_two_neighbour"):kf.index("test_get_grid_spacing")]
    out["rho_array_one_neighbour"] = {"rho": [1e10, 1.2, 1.2], "velocity": _stream(one, "velocity"),
                                      "pressure": _stream(one, "pressure")}
    out["rho_array_two_neighbour"] = {"rho": [1.2, 1.2, 1.2], "velocity": _stream(two, "velocity"),
                                      "pressure": _stream(two, "pressure")}
    sp = kf[kf.index("test_spatderp3"):kf.index("window_generator")]
    out["spatderp3"] = {
        "dx": 0.4, "N": 128, "wlen": 32,
        "linspace": {"d1p": [-19.8, -0.2, 50], "d1v": [-20, 0, 51], "d3p": [20.2, 39.8, 50],
                     "d3v": [20, 40, 51], "d2p": [0.2, 19.8, 50], "d2v": [0, 20, 51]},
        "real_p": _stream(sp, "real_p"), "imag_p": _stream(sp, "imag_p"),
        "real_v": _stream(sp, "real_v"), "imag_v": _stream(sp, "imag_v"),
        "window": _stream(sp, "window"),
    }
    wg = kf[kf.index("window_generator"):]
    out["window_generator"] = {"W": 32, "patch_error": 70, "values": _stream(wg, "window_verify")}

    # test/Kernel/WisdomCache.cpp
    checks = re.findall(r"is_approx\(discr1\.([a-z_]+)(?:\.(real|imag)\(\))?\.coeff\((\d+)\),\s*([-+\d.eE]+)\)", wc)
    out["wisdom_cache"] = {"dx": 0.2, "N": 115,
                           "checks": [[f, part or "", int(i), float(v)] for f, part, i, v in checks]}

    # test/Kernel/Domain.cpp
    init = dm[dm.index("test_initial_values"):]
    out["speaker_initial_values"] = {
        "domain_size_world": [50, 60], "dx": 0.2, "speaker": [4.1, 5.1],
        "p0_25_20": float(re.search(r"p0\(25, 20\),\s*([\d.]+)\)", init).group(1)),
        "p0_24_20": float(re.search(r"is_approx\(domain->current_values\.p0\(24, 20\),\s*([\d.]+)\)", init).group(1)),
    }
    cnt = re.search(r"domain_list\.size\(\),\s*1 \+ 4 \+ 4\)", dm)
    out["domain_scene"] = {"n_domains": 9 if cnt else None, "size_x": 250, "bottom_right_y": 300,
                           "air_neighbours_without_pml": 0, "air_neighbours_with_pml": 4,
                           "edges": {"T": 0, "B": 0.25, "L": 0.35, "R": 0.7}, "L_lr": True}

    # test/Kernel/Scene.cpp
    out["scene_pml"] = {"size_world": [40, 60], "alpha": 0.1, "pml_cells": 50,
                        "n_domains": 9, "n_pml": 8, "n_secondary": 4}
    assert "1 + 4 + 4" in sc and "4 + 4" in sc
    return out


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    data = main(ref)
    path = os.path.join(HERE, "reference_kats.json")
    with open(path, "w") as f:
        json.dump(data, f, indent=1)
    print("wrote", path)
