// ErrorLatencyProfile.hpp — sizing the number of estimators (the reference's
// include/ErrorLatencyProfile.hpp interface).  ErrorProfile runs the reference's regression
// procedure with its 2^14 + 1 calculate() calls batched into two device launches
// (zg_run_groups, zg_run); TimeProfile doubles calculate() calls under a time budget.
#ifndef ERROR_LATENCY_PROFILE
#define ERROR_LATENCY_PROFILE

#include <assert.h>
#include <math.h>

#include <string>

#include "Time.hpp"
#include "Type.hpp"
#include "ZGraphInstance.hpp"

template <typename EdgeData>
class TimeProfile {
 private:
  unsigned long long num_finished_estimators;
  double current_estimation;
  void reset();
  void update(unsigned long long new_num_estimators, double new_estimation);

 public:
  double run(ZGraphInstance<EdgeData>& zgraph_instance, VertexId num_vertices_in_pattern, unsigned int time_limit);
};

template <typename EdgeData>
class ErrorProfile {
 private:
  double calculate_bound(double epsilon, double delta, double num_sample_edge_calls,
                         double num_conditional_sample_edge_call, double estimation, EdgeId max_degree,
                         EdgeId num_edges);

 public:
  double run(ZGraphInstance<EdgeData>& zgraph_instance, VertexId num_vertices_in_pattern, double required_error_rate,
             double required_confidence, Estimation& init_estimation);
  unsigned long long get_num_estimators(ZGraphInstance<EdgeData>& zgraph_instance, VertexId num_vertices_in_pattern,
                                        double required_error_rate, double required_confidence);
};

#endif
