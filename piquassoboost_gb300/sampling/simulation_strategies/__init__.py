"""Drop-in boson-sampling strategies (the reference's
piquassoboost.sampling.simulation_strategies API, generalised Clifford &
Clifford B forms) over the GPU pmf layers."""
