"""Command line front-end: ``python -m bqa_gb300.cli -i job.json -o result.json -l INFO``.

Same interface as the reference's ``bqa_cli`` (``src/bqa/cli.py``): the job config as JSON on
``-i/--input`` (stdin if absent), the result list as JSON on ``-o/--output`` (stdout if
absent), a logging level on ``-l/--log-level``; on any error the chain of causes goes to
stderr and the exit code is 1.  JSON has no tuple keys, so edges and nodes come as lists:
``"edges": [[[0, 1], 1.0], ...]``, ``"nodes": [[0, 0.3], ...]`` (the reference DSL accepts
both forms).

Results are written as they are produced from numpy arrays -- no per-qubit Python lists --
so a 200k-qubit Bloch-vector result streams out in well under a second.
"""
from __future__ import annotations

import io
import json
import logging
import os
import sys
from pathlib import Path

LOG_LEVELS = ["DEBUG", "INFO", "WARNING", "ERROR"]
DEFAULT_LOG_LEVEL = "INFO"


class CliError(Exception):
    pass


def _usage(prog: str) -> str:
    return (f"usage: {prog} [options]\n\n"
            "    -i | --input  [PATH]          path to a *.json job config (stdin if absent)\n"
            "    -o | --output [PATH]          path to the *.json result (stdout if absent)\n"
            f"    -l | --log-level [LEVEL]      one of {', '.join(LOG_LEVELS)} ({DEFAULT_LOG_LEVEL} if absent)\n"
            "    -h | --help                   show this message and exit")


def _json_path(path: str) -> Path:
    p = (Path(os.getcwd()) / Path(path)).resolve()
    if p.suffix != ".json":
        raise CliError(f"{p} must have .json suffix")
    return p


def parse_args(argv: list[str]) -> dict:
    """Options of ``argv`` (argv[0] is the program); exits 0 on --help, 1 on an unknown option."""
    ctx = {"input": None, "output": None, "log-level": DEFAULT_LOG_LEVEL}
    args = iter(argv[1:])
    for arg in args:
        if arg in ("-h", "--help"):
            print(_usage(argv[0]))
            sys.exit(0)
        key = {"-i": "input", "--input": "input", "-o": "output", "--output": "output",
               "-l": "log-level", "--log-level": "log-level"}.get(arg)
        if key is None:
            print(f"Invalid command line argument {arg}, run `{argv[0]} --help` to get the documentation")
            sys.exit(1)
        val = next(args, None)
        if val is None:
            raise CliError(f"{'Logging level' if key == 'log-level' else key.capitalize() + ' file'} "
                           f"is not provided after {arg} key")
        if key == "log-level":
            if val not in LOG_LEVELS:
                raise CliError(f"{val} cannot be interpeted as a logging level, must be one of {', '.join(LOG_LEVELS)}")
            ctx[key] = val
        else:
            ctx[key] = _json_path(val)
    return ctx


def read_config(src) -> dict:
    try:
        if src is None:
            return json.load(sys.stdin)
        with open(src) as f:
            return json.load(f)
    except (json.JSONDecodeError, UnicodeError, OSError) as e:
        raise CliError("Error while parsing json data") from e


def write_results(results: list, dst: io.TextIOBase) -> None:
    """Stream ``[[kind, values], ...]`` as JSON; numpy arrays are written row by row."""
    dst.write("[")
    for k, (kind, values) in enumerate(results):
        dst.write(", " if k else "")
        dst.write(f"[{json.dumps(kind)}, ")
        if hasattr(values, "ndim") and values.ndim == 2:
            dst.write("[")
            rows = values.tolist()
            for i, row in enumerate(rows):
                dst.write((", [" if i else "[") + ", ".join(repr(float(v)) for v in row) + "]")
            dst.write("]")
        elif hasattr(values, "ndim"):
            dst.write("[" + ", ".join(str(int(v)) for v in values.tolist()) + "]")
        else:
            dst.write(json.dumps(values))
        dst.write("]")
    dst.write("]")


def format_error(e: BaseException) -> str:
    msgs = []
    while e is not None:
        msgs.append(str(e))
        e = e.__cause__
    return "\ncaused by: ".join(msgs)


def main(argv: list[str] | None = None) -> int:
    argv = sys.argv if argv is None else argv
    try:
        ctx = parse_args(argv)
        logging.basicConfig(level=getattr(logging, ctx["log-level"]),
                            format="%(asctime)s [%(levelname)s] %(message)s", datefmt="%Y-%m-%d %H:%M:%S")
        config = read_config(ctx["input"])
        from .core import run_qa
        results = run_qa(config, as_arrays=True)
        try:
            if ctx["output"] is None:
                write_results(results, sys.stdout)
                sys.stdout.write("\n")
            else:
                with open(ctx["output"], "w") as f:
                    write_results(results, f)
        except OSError as e:
            raise CliError("Error while writing result") from e
    except Exception as e:  # the reference reports every failure the same way
        print(format_error(e), file=sys.stderr)
        return 1
    return 0


if __name__ == "__main__":
    sys.exit(main())
