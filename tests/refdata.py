"""Where the reference's test cases are, for the tests that compare the
shipped data and the restart reader with the reference's own files.

IZEM_REFERENCE_TESTCASES names the reference's ``devel-izem/testcases``
directory; without it those tests are skipped.  There is no default path."""
import os

import pytest

TESTCASES = os.environ.get("IZEM_REFERENCE_TESTCASES", "")

needs_reference = pytest.mark.skipif(not (TESTCASES and os.path.isdir(TESTCASES)),
                                     reason="IZEM_REFERENCE_TESTCASES does not name the reference's testcases directory")


def path(*parts):
    return os.path.join(TESTCASES, *parts)
