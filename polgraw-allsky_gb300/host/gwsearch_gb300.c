/* gwsearch-gb300: drop-in for the reference network search program
 * (search/network/src-cpu/main.c:37-155) with job_core() on the GPU. */
#include "../../include/polgraw_gb300_host.h"

int main(int argc, char *argv[]) { return pa_host_main(argc, argv); }
