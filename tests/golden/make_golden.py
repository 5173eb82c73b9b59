"""Regenerate tests/golden/params_reference.json by importing the reference's own params.i
parser (read_params.py:1-228) from the reference checkout.  Run in the build container only:
    python tests/golden/make_golden.py /path/to/reference
The reference is not available where the tests run; the JSON is the committed fixture."""
import json
import os
import sys

ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SPARC_REFERENCE", "")
sys.path.insert(0, ref)
import read_params  # noqa: E402

out = {
    "params_i": open(os.path.join(ref, "params.i")).read(),
    "get_nx": read_params.get_nx(),
    "get_nz": read_params.get_nz(),
    "get_xlength": read_params.get_xlength(),
    "get_dt": read_params.get_dt(),
    "get_dt_simulation": read_params.get_dt_simulation(),
    "get_total_simulation_time": read_params.get_total_simulation_time(),
    "get_solarmodel": read_params.get_solarmodel(),
    "get_excitedepth": read_params.get_excitedepth(),
    "get_obs_depth": read_params.get_obs_depth(),
    "get_directory": read_params.get_directory(),
}
with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "params_reference.json"), "w") as f:
    json.dump(out, f, indent=1)
print({k: v for k, v in out.items() if k != "params_i"})
