// Included inside namespace evolving_graphs::util by util/cpu_topology.h.
enum { NUM_SOCKET = 1, NUM_PHYSICAL_CPU_PER_SOCKET = 1, SMT_LEVEL = 1 };
const int OS_CPU_ID[1][1][1] = {{{0}}};
