"""Loader of tests/golden/reference_sampler.json (the reference's seeded
boson samples) for the sampler tests."""
import json
import os

import numpy as np

_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_sampler.json")


def load():
    with open(_PATH) as f:
        d = json.load(f)
    for c in d["seeding_cases"] + d["sequences"]:
        m = c["modes"]
        c["U"] = np.array([complex(a, b) for a, b in c["interferometer"]]).reshape(m, m)
    return d
