"""The bench.py commands quoted in profiles/*.md parse with bench.py's own
command line, every summary quotes at least one, and a summary named for a
workload (c2_64cube, c3_256bodies, c5_64bodies) runs that workload: the
default workload of bench.py is the 256-body batch, so a C2 or C5 command
must name its own."""
import glob
import os
import re
import shlex
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

WORKLOAD_OF = {"_c2_64cube": "c2", "_c3_256bodies": "c3", "_c5_64bodies": "c5"}


def bench_commands(text):
    """The argument lists after each `python bench.py` (continuation lines
    joined; a command ends at a redirection, `&&` or a pipe)."""
    text = text.replace("\\\n", " ")
    for line in text.splitlines():
        for part in line.split("python bench.py")[1:]:
            part = re.split(r"\s(?:>|2>|&&|\|)\s", " " + part + " ")[0]
            yield shlex.split(part)


def test_profile_commands_parse_and_name_their_workload():
    import bench
    ap = bench.make_parser()
    files = sorted(glob.glob(os.path.join(ROOT, "profiles", "*.md")))
    assert files
    for f in files:
        cmds = list(bench_commands(open(f).read()))
        assert cmds, "%s quotes no bench.py command" % os.path.basename(f)
        want = next((w for k, w in WORKLOAD_OF.items() if k in os.path.basename(f)), None)
        for argv in cmds:
            args = ap.parse_args(argv)
            if want:
                assert args.workload == want, (os.path.basename(f), argv)
