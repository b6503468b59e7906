"""Writes tests/golden/tutorials/<name>.json from picFoam's tutorial case
directories (TEST INFRASTRUCTURE; run where picFoam's tree is present):

    PICFOAM_TUTORIALS=<picFoam source>/tutorials python tests/golden/make_tutorial_cases.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

from picfoam_gb300 import ofcase  # noqa: E402
import tutorial_cases  # noqa: E402

# name -> loaded with its unmapped entries listed (not refused)
TUTORIALS = {"plasmaOscillation": False, "thermalization": False, "thermalization_binaryCollision": False,
             "ionization": False, "magneticRotation": False, "rlcCircuit": False, "floatingBoundary": True,
             "electricAcceleration": True}


# fixture -> (tutorial, IonizationModel override)
VARIANTS = {"thermalization_perez": ("thermalization", "Perez")}


def main():
    root = os.environ.get("PICFOAM_TUTORIALS") or (sys.argv[1] if len(sys.argv) > 1 else None)
    if not root or not os.path.isdir(root):
        raise SystemExit("set PICFOAM_TUTORIALS to picFoam's tutorials directory")
    out = os.path.join(HERE, "tutorials")
    os.makedirs(out, exist_ok=True)
    for name, allow in TUTORIALS.items():
        case = ofcase.load_case(os.path.join(root, name), allow_unsupported=allow)
        with open(os.path.join(out, name + ".json"), "w") as f:
            json.dump(tutorial_cases.dump(case), f, indent=1)
        print(name, "unmapped:", case.unsupported)
    # the thermalization tutorial carries PerezIonizationCoeffs for argon with
    # the model switched off; this fixture switches it on
    for name, (src, model) in VARIANTS.items():
        case = ofcase.load_case(os.path.join(root, src), ionization_model=model)
        with open(os.path.join(out, name + ".json"), "w") as f:
            json.dump(tutorial_cases.dump(case), f, indent=1)
        print(name, "unmapped:", case.unsupported)


if __name__ == "__main__":
    main()
