#!/usr/bin/env bash
# Builds oracle/_ref/ref_golden from the reference's own math headers, where they lie.
# TEST INFRASTRUCTURE ONLY: it runs where a reference checkout exists, named by the
# AXIOM_REFERENCE environment variable (required); outputs go only to oracle/_ref/
# (git-ignored).
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${AXIOM_REFERENCE:?set AXIOM_REFERENCE to the reference checkout}"
if [ ! -d "$REF/include/axiom/math" ]; then
    echo "reference checkout not found at $REF" >&2
    exit 2
fi
mkdir -p "$HERE/_ref"
g++ -std=c++20 -O2 -ffp-contract=off -I "$REF/include" "$HERE/ref_golden.cpp" -o "$HERE/_ref/ref_golden"
echo "$HERE/_ref/ref_golden"
