// NetworkInterface.hpp — process-level set-up.  The reference runs one MPI rank per node; here one
// process drives one GPU, so this is a single "partition" and the MPI calls applications make
// directly (MPI_Barrier) are local no-ops.  zg_init selects the device.
#ifndef NETWORK_INTERFACE
#define NETWORK_INTERFACE

#include <assert.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include <iostream>

#ifndef MPI_VERSION
typedef int MPI_Comm;
#define MPI_COMM_WORLD 0
static inline int MPI_Barrier(MPI_Comm) { return 0; }
#endif

enum MessageTag { TransferSeed, ShuffleGraph, ReduceEstimation };

class NetworkInterface {
 private:
  static NetworkInterface* instance;
  int partition_id;
  int partitions;
  NetworkInterface(int* argc, char*** argv);
  ~NetworkInterface();

 public:
  static void init_network_interface(int* argc, char*** argv);
  static NetworkInterface* get_instance(int* argc = nullptr, char*** argv = nullptr);
  static void finalize_instance();
  void pause();
  int get_partition_id();
  int get_num_partitions();
};

#endif
