#!/usr/bin/env bash
# Builds the CPU restatement (oracle/vdbscan_oracle.c) into
# oracle/_build/liborc_vdbscan.so.  Test infrastructure only.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
mkdir -p "$HERE/_build"
"${CC:-gcc}" -O2 -std=c11 -ffp-contract=off -fopenmp -shared -fPIC -Wall -Wextra \
  "$HERE/vdbscan_oracle.c" -o "$HERE/_build/liborc_vdbscan.so" -lm
echo "built $HERE/_build/liborc_vdbscan.so"
