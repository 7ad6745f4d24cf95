"""Command line of the GB300 PSTD solve, mirroring openPSTD's CLI
(CLI/main.cpp): ``create`` writes the default scene (CreateDefaultConf),
``run -g`` runs a scene on the GPU (RunCommand, CLI/main.cpp:365-464) and
stores the results in the layout of the reference's HDF5 export
(shared/export/HDF5Export.cpp:41-74): ``frame/<domain>/<frame>`` arrays of
shape (Nx, Ny) filled in the kernel's row-major (x fastest) order, and
``receiver/<r>`` series.  Scenes are JSON files of the PSTDConfiguration
fields, with results in a NumPy ``.npz`` archive with those keys, or the
reference's own scene files (``.pstd``, shared/PSTDFile.cpp), whose results
go back into the file as RunCommand stores them (frames per domain, receiver
samples appended).  ``.pstd`` files need the unqlite library the reference
builds (``--unqlite-lib`` or ``PSTD_UNQLITE_LIB``).

    python -m openpstd_gb300 create scene.json|scene.pstd
    python -m openpstd_gb300 run -g scene.json -o results.npz [--save-nth N] [--stride S]
    python -m openpstd_gb300 run -g scene.pstd
"""
from __future__ import annotations

import argparse
import sys

import numpy as np


def _is_pstd(path: str) -> bool:
    return str(path).lower().endswith(".pstd")


def _create(args) -> int:
    from .config import PSTDConfiguration
    if _is_pstd(args.scene_file):
        from .pstdfile import PSTDFile
        PSTDFile.New(args.scene_file, args.unqlite_lib).close()   # version, default scene, empty results
    else:
        PSTDConfiguration.CreateDefaultConf().save(args.scene_file)
    print(f"wrote the default scene to {args.scene_file}")
    return 0


def run_into_file(path: str, kernel, output_base=None, unqlite_lib=None, log=print) -> int:
    """RunCommand on a scene file (CLI/main.cpp:419-449): open it, take its
    scene, delete old results, initialise new ones, run `kernel` (an object
    with the KernelInterface methods) with an output that stores every frame
    (SaveNextResultsFrame) and receiver sample (SaveReceiverData) in the file,
    then commit.  Returns the number of frames stored."""
    from .kernel import KernelCallback
    from .pstdfile import PSTDFile
    f = PSTDFile.Open(path, unqlite_lib)
    try:
        conf = f.GetSceneConf()
        log("Delete old results(if any)")
        f.DeleteResults()
        log("initilize new results")
        f.InitializeResults()
        stored = [0]
        base = output_base or KernelCallback

        class FileOutput(base):
            # CLIOutput (CLI/output.cpp:30-39)
            def WriteFrame(self, frame, domain, data):
                f.SaveNextResultsFrame(domain, data)
                stored[0] += 1

            def WriteSample(self, start, receiver, data):
                f.SaveReceiverData(receiver, data)

        out = FileOutput()
        kernel.initialize_kernel(conf, out)
        kernel.run(out)
        f.Commit()
        return stored[0]
    finally:
        f.close()


def _run(args) -> int:
    from .config import PSTDConfiguration
    from .kernel import KernelCallback, PSTDKernel
    if not args.gpu_accelerated:
        print("error: this build provides the GPU solver only; run with -g", file=sys.stderr)
        return 1
    if args.multithreaded:
        print("warning: -m selects the reference's CPU solver; the GPU solver runs", file=sys.stderr)
    debug = args.debug
    if _is_pstd(args.scene_file):
        class Log(KernelCallback):
            def Info(self, message):
                if debug:
                    print(message)

            def Warning(self, message):
                print("warning:", message, file=sys.stderr)

            def Error(self, message):
                print("error:", message, file=sys.stderr)

        n = run_into_file(args.scene_file, PSTDKernel(GPU=True), Log, args.unqlite_lib)
        print(f"{n} frames stored in {args.scene_file}")
        return 0
    conf = PSTDConfiguration.load(args.scene_file)
    frames, samples = {}, {}
    stride = max(1, args.stride)

    class Output(KernelCallback):
        # CLIOutput (CLI/output.cpp:30-68): frames and samples go to the result store
        def WriteFrame(self, frame, domain, data):
            frames[(domain, frame)] = data

        def WriteSample(self, start, receiver, data):
            samples.setdefault(receiver, []).extend(data)

        def Info(self, message):
            if debug:
                print(message)

        def Debug(self, message):
            if debug:
                print(message)

        def Warning(self, message):
            print("warning:", message, file=sys.stderr)

        def Error(self, message):
            print("error:", message, file=sys.stderr)

    k = PSTDKernel(GPU=True)
    out = Output()
    k.initialize_kernel(conf, out)
    md = k.get_metadata()
    k.run(out, save_nth=args.save_nth, stride=stride)
    store = {}
    for (d, f), data in frames.items():
        nx, ny = md.DomainMetadata[d][0], md.DomainMetadata[d][1]
        store[f"frame/{d}/{f}"] = data.reshape((nx + stride - 1) // stride, (ny + stride - 1) // stride)
    for r, v in samples.items():
        store[f"receiver/{r}"] = np.asarray(v, np.float32)
    np.savez(args.output, **store)
    print(f"{len(frames)} frames, {len(samples)} receivers -> {args.output}")
    return 0


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m openpstd_gb300")
    sub = ap.add_subparsers(dest="command", required=True)
    c = sub.add_parser("create", help="write the default scene (CreateDefaultConf): JSON, or a .pstd file")
    c.add_argument("scene_file")
    c.add_argument("--unqlite-lib", default=None, help="unqlite shared library for .pstd files")
    r = sub.add_parser("run", help="run the PSTD algorithm on a scene")
    r.add_argument("scene_file")
    r.add_argument("-g", "--gpu-accelerated", action="store_true", help="use the GPU for the calculations")
    r.add_argument("-m", "--multithreaded", action="store_true", help="the reference's multi-threaded CPU solver")
    r.add_argument("-o", "--output", default="results.npz", help="result archive (HDF5-export layout)")
    r.add_argument("--save-nth", type=int, default=0, help="keep every n-th frame (0: the scene's SaveNth)")
    r.add_argument("--stride", type=int, default=1, help="keep every stride-th row and column of each frame")
    r.add_argument("--debug", action="store_true", help="show the kernel's log")
    r.add_argument("--unqlite-lib", default=None, help="unqlite shared library for .pstd files")
    args = ap.parse_args(argv)
    return _create(args) if args.command == "create" else _run(args)


if __name__ == "__main__":
    sys.exit(main())
