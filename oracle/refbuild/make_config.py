"""Writes the reference's generated configuration header for the pin build.

The reference's meson build turns apps/autogenerated/biocma_cst_config.hpp.in
into biocma_cst_config.hpp with the values of apps/autogenerated/meson.build
(conf_data, L26-L50; the CPU build's allocation factor 2.5, buffer ratio 1
and 1024 particles per team, L9-L24) and the project version of meson.build
(1.2.1).  This script performs the same substitution on the template read
from the reference tree, so the compiled headers see the reference's own
compile-time flags (event counter on, probes off).

    python make_config.py <reference root> <output header>
    python make_config.py --variant <reference root> <output header>
    python make_config.py --probe <reference root> <output header>

With --probe the configuration has the reference's probes on (use_probe =
true, its buffer of probe_buffer_size values), for the build of its cycle
whose probe records pin the oracle's.

With --variant it writes the model-variant header instead
(apps/autogenerated/variant_model.hxx, which the reference's
devutils/generate_model_loader.py fills with its model list): the container
variant over the two reference models the cycle pins run, FixedLength and
SimpleAcetate.
"""
import re
import sys

VALUES = {
    "probe_buffer_size": "10e3",
    "__f__redirect__": "false",
    "__f_verbose__": "true",
    "dump_particle_state": "true",
    "use_probe": "false",
    "const_number_simulation": "false",
    "default_particle_container_allocation_factor": "2.5",
    "MC_MAX_PARTICLE_BUFFER": "100e6",
    "debug_MC_RAND_DEFAULT_SEED": "2024",
    "_dead_particle_ratio_threshold": "0.01",
    "cma_data_folder_path": '"cma_data"',
    "enable_event_counter": "true",
    "shrink_ratio": "0.1",
    "default_MC_buffer_ratio": "1",
    "__f_compress_export__": "true",
    "__f_export_age__": "true",
    "default_particle_per_team_contributions": "1024",
    "default_particle_per_team_cycle": "1024",
    "default_particle_per_team_move": "1024",
    "default_particle_per_team_leave": "0",
    "result_dir_path": '"./results/"',
}
DEFINES = {"_BIOMC_VERSION_MAJOR": "1", "_BIOMC_VERSION_MINOR": "2", "_BIOMC_VERSION_DEV": "1",
           "_BIOMC_BUILD_MODE": '"release"'}


def main(ref_root: str, out: str, probes: bool = False) -> None:
    src = open(f"{ref_root}/apps/autogenerated/biocma_cst_config.hpp.in").read()
    values = dict(VALUES, use_probe="true") if probes else VALUES

    def mesondefine(m):
        name = m.group(1)
        return f"#define {name} {DEFINES[name]}"

    src = re.sub(r"#mesondefine\s+(\w+)", mesondefine, src)

    def at(m):
        name = m.group(1)
        if name not in values:
            raise KeyError(f"no value for @{name}@")
        return values[name]

    src = re.sub(r"@(\w+)@", at, src)
    with open(out, "w") as f:
        f.write(src)


MODELS = ("fixed_length", "FixedLength"), ("simple_acetate", "SimpleAcetate")


def variant(ref_root: str, out: str) -> None:
    src = open(f"{ref_root}/apps/autogenerated/variant_model.hxx").read()
    inc = "\n".join(f"#include <models/{h}.hpp>" for h, _ in MODELS)
    types = ", ".join(f"::MC::ParticlesContainer<::Models::{t}>" for _, t in MODELS)
    src = src.replace("@INCLUDES@", inc).replace("@VARIANT_TYPE@", types)
    with open(out, "w") as f:
        f.write(src)


if __name__ == "__main__":
    if sys.argv[1] == "--variant":
        variant(sys.argv[2], sys.argv[3])
    elif sys.argv[1] == "--probe":
        main(sys.argv[2], sys.argv[3], probes=True)
    else:
        main(sys.argv[1], sys.argv[2])
