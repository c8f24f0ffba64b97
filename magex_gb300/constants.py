"""Physical constants of the magex spin model (units: meV, tesla, ps, kelvin).

The values are those of magex ``magex/spinmodel.py:28-30``; the LLG step must use the same
numbers bit for bit, otherwise trajectories drift from the reference at the 1e-16 level every step.
"""
MU_B = 5.7883818060e-2      # Bohr magneton, meV / T
K_B = 8.617333262e-2        # Boltzmann constant, meV / K
GAMMA = 0.1760859630        # electron gyromagnetic ratio, rad / (ps T)
HBAR_MEV_PS = 0.6582119569   # reduced Planck constant, meV ps (magex/quantum.py:34)
