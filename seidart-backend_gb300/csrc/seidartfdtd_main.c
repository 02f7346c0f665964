/* seidartfdtd -- drop-in for the reference CLI (src/fortran/main.f08):
 *   seidartfdtd <input.json> [seismic=true|false] [density_method=...]
 * Reads input.json and the .dat inputs from the working directory, runs the
 * GPU solver and writes the per-step snapshots there. */
#include "../../include/seidart_gpu.h"

int main(int argc, char** argv) { return seidart_cli_main(argc, argv); }
