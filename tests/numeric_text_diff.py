"""Python 3 restatement of the reference's numeric text diff rule.

Follows kokkos/tests/tools/numeric_text_diff (Python 2 only upstream): two
whitespace-separated numeric text files match when every pair of differing
fields has relative error |a-b|/max(|a|,|b|) <= rel_tol, fields where both
magnitudes are <= floor being treated as equal (:61-88). Lines are paired by
position; the upstream tool pairs the '-'/'+' lines of `diff -u`, which is the
same pairing for files of equal length whose lines all changed in place.
"""
import argparse
import sys


def compare_lines(lines_a, lines_b, rel_tol=1e-3, floor=1e-6):
    """Returns a list of (line_no, line_a, line_b) that differ beyond tolerance."""
    if len(lines_a) != len(lines_b):
        raise ValueError("Files have differing line counts.")
    bad = []
    for i, (la, lb) in enumerate(zip(lines_a, lines_b)):
        fa, fb = la.split(), lb.split()
        if len(fa) != len(fb):
            raise ValueError("Number of fields differ for line %d" % (i + 1))
        for sa, sb in zip(fa, fb):
            if sa == sb:
                continue
            try:
                va, vb = float(sa), float(sb)
            except ValueError:
                bad.append((i + 1, la, lb))
                break
            if abs(va) > floor or abs(vb) > floor:
                rel = abs(va - vb) / max(abs(va), abs(vb))
                if rel > rel_tol:
                    bad.append((i + 1, la, lb))
                    break
    return bad


def compare_files(path_a, path_b, rel_tol=1e-3, floor=1e-6):
    with open(path_a) as fa, open(path_b) as fb:
        return compare_lines(fa.read().splitlines(), fb.read().splitlines(), rel_tol, floor)


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--relative-tolerance", type=float, default=1e-3)
    p.add_argument("--floor", type=float, default=1e-6)
    p.add_argument("file1")
    p.add_argument("file2")
    a = p.parse_args(argv)
    try:
        bad = compare_files(a.file1, a.file2, a.relative_tolerance, a.floor)
    except ValueError as e:
        print(e)
        return 1
    if bad:
        print("Files differ with relative_tol=%g & floor=%g:" % (a.relative_tolerance, a.floor))
        for n, la, lb in bad[:20]:
            print("%d\n-%s\n+%s" % (n, la, lb))
        return 1
    print("Files are the same.")
    return 0


if __name__ == "__main__":
    sys.exit(main())
