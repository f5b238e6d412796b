// cli_main.cpp -- the oracle's `probebwa` executable (test infrastructure):
// src/main.rs restated over the CPU oracle, the reference side of the
// command-line parity tests.
#include "oracle.h"

int main(int argc, char** argv) { return orc_cli_main(argc, argv); }
