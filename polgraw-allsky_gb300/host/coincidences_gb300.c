/* coincidences-gb300: drop-in for the reference coincidence program
 * (coincidences/src/coincidences.c) with the coincidence step on the GPU. */
#include "../../include/polgraw_gb300_host.h"

int main(int argc, char *argv[]) { return pa_coinc_main(argc, argv); }
