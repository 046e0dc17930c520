"""Writes tests/golden/reference_cases/<example>.json: the case dictionary
that each of the reference's example scripts (examples/<example>/case.py in
the MicroFC project) prints.  Run in a checkout that has the reference next
to it; the fixtures are committed, so the tests do not need the reference.

    python tests/golden/make_reference_cases.py /path/to/MicroFC
"""
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main(reference: str) -> None:
    out_dir = os.path.join(HERE, "reference_cases")
    os.makedirs(out_dir, exist_ok=True)
    examples = os.path.join(reference, "examples")
    for name in sorted(os.listdir(examples)):
        script = os.path.join(examples, name, "case.py")
        if not os.path.isfile(script):
            continue
        text = subprocess.run([sys.executable, script], capture_output=True, text=True, check=True,
                              cwd=os.path.dirname(script)).stdout
        d = json.loads(text)
        with open(os.path.join(out_dir, name + ".json"), "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
            f.write("\n")
        print(name, len(d), "keys")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
