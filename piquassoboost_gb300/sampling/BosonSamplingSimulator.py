"""Drop-in for the reference's BosonSamplingSimulator
(piquassoboost/sampling/BosonSamplingSimulator.py): runs a simulation
strategy for a number of samples."""


class BosonSamplingSimulator:
    def __init__(self, simulation_strategy):
        self.simulation_strategy = simulation_strategy

    def get_classical_simulation_results(self, input_state, samples_number: int = 1):
        return self.simulation_strategy.simulate(input_state, samples_number)
