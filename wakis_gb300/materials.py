"""Material library (same keys and values as wakis/materials.py:28-41).

Format: 'key': [eps_r, mu_r] or [eps_r, mu_r, sigma (S/m)]; eps = eps_r*eps_0.
"""

import numpy as np

material_lib = {
    "pec": [np.inf, 1.0],
    "vacuum": [1.0, 1.0],
    "dielectric": [10.0, 1.0],
    "lossy metal": [10, 1.0, 10],
    "copper": [5.8e07, 1.0, 5.8e07],
    "berillium": [2.5e07, 1.0, 2.5e07],
    "stainless steel": [1.4e06, 1.0, 1.4e06],
}

material_colors = {
    "pec": "white",
    "vacuum": "tab:blue",
    "dielectric": "tab:green",
    "lossy metal": "tab:orange",
    "copper": [0.82745099, 0.698039, 0.49019599],
    "berillium": [0.82745099, 0.698039, 0.49019599],
    "stainless steel": "silver",
    "martensite": [0.0, 1.0, 1.0],
    "other": "cyan",
}
