"""Repository hygiene (CPU): the committed summaries under profiles/ cite
only commands that run committed files, and product sources name neither
working folders nor this machine's paths."""
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_profiles_cite_committed_commands_only():
    for p in glob.glob(os.path.join(ROOT, "profiles", "*.md")):
        txt = open(p).read()
        assert "_work/" not in txt and "/root/" not in txt, p
        for cmd in re.findall(r"python (\S+\.py)", txt):
            assert os.path.exists(os.path.join(ROOT, cmd)), (p, cmd)


def test_sources_name_no_working_paths():
    pats = ("_work/", "/root/", "gpurun")
    files = glob.glob(os.path.join(ROOT, "singularity-eos_gb300", "csrc", "*"))
    files += glob.glob(os.path.join(ROOT, "include", "*"))
    files += [os.path.join(ROOT, "bench.py"), os.path.join(ROOT, "__graft_entry__.py")]
    for f in files:
        txt = open(f, errors="replace").read()
        for s in pats:
            assert s not in txt, (f, s)
