#!/bin/sh
# Builds the CPU FP64 oracle (test infrastructure only) into oracle/libvk_oracle.so.
set -e
here=$(cd "$(dirname "$0")" && pwd)
${CC:-gcc} -O2 -std=c11 -fPIC -shared -fopenmp -fno-fast-math -ffp-contract=off \
  -o "$here/libvk_oracle.so" "$here/vk_oracle.c" -lm
