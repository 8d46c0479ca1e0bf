"""Records the agreement fractions of the GPU parity tests: with LGB_PARITY_LOG set to a file path, each
comparison appends one JSON line (test id, fraction of samples or pixels within tolerance, the tolerance). The
fractions of samples that differ are the rare branch flips the parity tests allow; this is how they are measured."""
import json
import os


def record(fraction, rtol):
    path = os.environ.get("LGB_PARITY_LOG")
    if not path:
        return
    test = os.environ.get("PYTEST_CURRENT_TEST", "?").split(" ")[0]
    with open(path, "a") as f:
        f.write(json.dumps({"test": test, "fraction": float(fraction), "rtol": rtol}) + "\n")
