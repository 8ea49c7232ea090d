#!/usr/bin/env python3
"""Run the reference's own test programs against the CPU oracle (and, for the programs
that need no GPU, against the product library too).

TEST INFRASTRUCTURE ONLY.  `make -C oracle reftests` compiles the reference's test
programs (test/pack/pack.c, test/iov/iov.c and test/flatten/flatten.c with test/dtpools,
test/simple/*.c) from the reference tree against liboracle_yaksa.so into oracle/_ref/,
and iov.c, lbub.c and test_contig.c against yaksa_gb300/lib/libyaksa.so as *_product.
This script runs them over the same matrix the reference generates for its
`make testing` target (maint/gentests.py:16-154: counts {17, 1075, 65536}, base types
{int, short_int, int:3+float:2, int:3+double:2, c_complex, c_double_complex}, segments
{1, 64}, orderings, overlaps, plus the -num-threads 4 and -blocking variants) and writes
a one-line-per-run summary.

The reference's pack test checks every result against closed-form arithmetic
progressions (test/dtpools/src/dtpools_init_verify.c), so a clean run pins the oracle's
type constructors, partial-element packing and operators to the reference.  The iov
test copies through the segment lists of two types with one signature and checks the
destination, which pins yaksa_iov and yaksa_iov_len; the flatten test packs with a type
and unpacks with its flattened-and-unflattened copy.

    python3 oracle/run_reftests.py [--iters-scale 0.25] [--out tests/golden/reftests_oracle.txt]
"""
import argparse
import os
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
REF_BIN = os.path.join(HERE, "_ref")

COUNTS = [17, 1075, 65536]
ITERS = {17: 32768, 1075: 128, 65536: 32}
TYPES = ["int", "short_int", "int:3+float:2", "int:3+double:2", "c_complex", "c_double_complex"]
OPLIST = {"int": "int", "short_int": "int", "int:3+float:2": "float",
          "int:3+double:2": "float", "c_complex": "complex", "c_double_complex": "complex"}


def pack_matrix(extra="", oplist=True, seed=1):
    """Yield argument strings in the order the reference's generator emits them."""
    for overlap in ["none", "regular", "irregular"]:
        for ordering in ["normal", "reverse", "random"]:
            if overlap != "none" and ordering != "normal":
                continue
            for segment in [1, 64]:
                if segment == 1 and (ordering != "normal" or overlap != "none"):
                    continue
                for count in COUNTS:
                    for t in TYPES:
                        ops = f" -oplist {OPLIST[t]}" if oplist else ""
                        yield (f"-datatype {t} -count {count} -seed {seed} -iters {{iters}} "
                               f"-segments {segment} -ordering {ordering} -overlap {overlap}"
                               f"{ops}{extra}", count)
                        seed += 1


def flatten_matrix(extra="", seed=1):
    for count in COUNTS:
        for t in TYPES:
            yield f"-datatype {t} -count {count} -seed {seed} -iters {{iters}}{extra}", count
            seed += 1


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--iters-scale", type=float, default=1.0)
    ap.add_argument("--variants", default="plain,threads,blocking")
    ap.add_argument("--out", default=None)
    ap.add_argument("--timeout", type=int, default=1800)
    args = ap.parse_args()

    lines = []
    failures = 0
    for prog in ["simple_test", "threaded_test", "lbub", "test_contig", "lbub_product",
                 "test_contig_product"]:
        t0 = time.time()
        r = subprocess.run([os.path.join(REF_BIN, prog)], capture_output=True, text=True,
                           timeout=args.timeout)
        ok = r.returncode == 0 and not r.stderr.strip() and not r.stdout.strip()
        failures += not ok
        lines.append(f"{'PASS' if ok else 'FAIL'} {prog} ({time.time() - t0:.2f}s)")
        print(lines[-1], flush=True)

    extras = {"plain": "", "threads": " -num-threads 4", "blocking": " -blocking"}
    for v in args.variants.split(","):
        for argstr, count in pack_matrix(extras[v]):
            iters = max(1, int(ITERS[count] * args.iters_scale))
            a = argstr.format(iters=iters)
            t0 = time.time()
            r = subprocess.run([os.path.join(REF_BIN, "pack")] + a.split(), capture_output=True,
                               text=True, timeout=args.timeout)
            ok = r.returncode == 0
            failures += not ok
            lines.append(f"{'PASS' if ok else 'FAIL'} pack {a} ({time.time() - t0:.2f}s)")
            print(lines[-1], flush=True)
            if not ok:
                print(r.stdout[-2000:], r.stderr[-2000:])

    def run(prog, a):
        nonlocal failures
        t0 = time.time()
        r = subprocess.run([os.path.join(REF_BIN, prog)] + a.split(), capture_output=True,
                           text=True, timeout=args.timeout)
        ok = r.returncode == 0
        failures += not ok
        lines.append(f"{'PASS' if ok else 'FAIL'} {prog} {a} ({time.time() - t0:.2f}s)")
        print(lines[-1], flush=True)
        if not ok:
            print(r.stdout[-2000:], r.stderr[-2000:])

    # segment lists: the oracle and the product; seeds continue where the generator's
    # pack lists end (4 pack lists of 108 runs)
    for extra in ("", " -num-threads 4"):
        for prog in ("iov", "iov_product"):
            for argstr, count in pack_matrix(extra, oplist=False, seed=433):
                run(prog, argstr.format(iters=max(1, int(ITERS[count] * args.iters_scale))))
    for extra in ("", " -num-threads 4"):
        for argstr, count in flatten_matrix(extra, seed=649):
            run("flatten", argstr.format(iters=max(1, int(ITERS[count] * args.iters_scale))))

    summary = f"{len(lines) - failures}/{len(lines)} passed"
    print(summary)
    if args.out:
        with open(args.out, "w") as f:
            f.write("# reference test programs run against the CPU oracle, and the ones "
                    "that need no GPU against the product (oracle/run_reftests.py)\n")
            f.write(f"# iters-scale {args.iters_scale}; host {os.uname().machine}\n")
            f.write("\n".join(lines) + "\n" + summary + "\n")
    return 1 if failures else 0


if __name__ == "__main__":
    sys.exit(main())
