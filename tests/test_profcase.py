"""The profiling cases that the summaries under profiles/ name (python -m distpca_gb300.profcase ...):
every case the summaries cite exists, and an unknown case is refused before any GPU work."""
import io
import re
import os
from contextlib import redirect_stderr

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cited_cases_exist():
    from distpca_gb300 import profcase

    cited = set()
    for name in os.listdir(os.path.join(ROOT, "profiles")):
        if name.endswith(".md"):
            text = open(os.path.join(ROOT, "profiles", name)).read()
            cited.update(re.findall(r"python -m distpca_gb300\.profcase ((?:[a-z]+ ?)+)", text))
    cases = {c for group in cited for c in group.split()}
    assert cases, "the summaries name no profiling case"
    assert cases <= set(profcase.CASES), cases - set(profcase.CASES)


def test_unknown_case_refused():
    from distpca_gb300 import profcase

    err = io.StringIO()
    with redirect_stderr(err):
        assert profcase.main(["no_such_case"]) == 2
    assert "unknown case" in err.getvalue()
