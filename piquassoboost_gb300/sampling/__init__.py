"""Drop-in permanent calculators (the reference's piquassoboost.sampling API)."""
