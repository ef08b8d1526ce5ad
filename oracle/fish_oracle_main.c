/* fish_oracle_main.c -- command-line front end of the CPU oracle (test
   infrastructure): takes fish's flags, prints fish's report lines. */
#include "fish_oracle.h"

int main(int argc, char **argv) { return or_fish_main(argc - 1, (const char **)(argv + 1)); }
