#!/bin/sh
# Builds the oracle (test infrastructure) as oracle/liboracle.so.  -ffp-contract=off keeps every FP64 operation
# unfused so x86 and Arm hosts produce the same bits; -O2 without -ffast-math keeps IEEE semantics.
set -e
cd "$(dirname "$0")"
${CXX:-g++} -std=c++17 -O2 -ffp-contract=off -fno-fast-math -fPIC -shared -Wall -Wno-unused-function \
    -o liboracle.so oracle.cpp -pthread
