"""`python -m parmec_gb300 deck.py [args]` runs an input deck like `parmec8 deck.py` (main.cpp:37-69)."""
import sys

from .parmec import run_deck


def main():
    if len(sys.argv) < 2:
        print("SYNOPSIS: python -m parmec_gb300 path/to/file.py")
        return 1
    run_deck(sys.argv[1], sys.argv[2:])
    return 0


if __name__ == "__main__":
    sys.exit(main())
