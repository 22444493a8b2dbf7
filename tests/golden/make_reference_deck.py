"""Writes tests/golden/bubbin_reference_deck1: the first deck of the reference's own
`bubbin` input file (the deck READINI reads, electric.f:275-337: k, nd(1..k), dt tfinal
nplot, cap bondx bondy E0, then one line per drop), taken verbatim from the reference
checkout. Run once where the reference is available; the GPU tests read the fixture.

    python tests/golden/make_reference_deck.py /path/to/ElectricBubbles/bubbin
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def first_deck(lines):
    k = int(lines[0].split()[0])
    return lines[:4 + k]


def main(path):
    with open(path) as f:
        lines = [ln.rstrip("\n") for ln in f]
    deck = first_deck(lines)
    out = os.path.join(HERE, "bubbin_reference_deck1")
    with open(out, "w") as f:
        f.write("\n".join(deck) + "\n")
    print("wrote %s (%d drops)" % (out, int(deck[0].split()[0])))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference/bubbin")
