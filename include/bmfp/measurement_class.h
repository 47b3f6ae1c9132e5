// Drop-in replacement for the reference's common/measurement_class.h.
//
// measurement_class keeps a format name, an elapsed time in seconds, the
// effective bandwidth (bytes / (elapsed * 1e9), GB/s) and the computational
// throughput (operations / (elapsed * 1e9), GFLOP/s); operator+= accumulates
// runs and finalize() turns the sums into means (measurement_class.h:9-56,
// measurement_class.cpp:7-16). compare_results reports, on stderr, a relative
// squared error sum((a-b)^2)/sum(b^2) above 1e-9 and the first entry that
// differs by more than 1e-8, and never aborts (measurement_class.h:58-87).
#ifndef BMFP_MEASUREMENT_CLASS_H
#define BMFP_MEASUREMENT_CLASS_H

#include <cmath>
#include <iostream>
#include <string>
#include <utility>

class measurement_class
{
  const size_t giga = 1000000000;

public:
  measurement_class () = default;
  measurement_class (std::string format, double elapsed_arg, double load_store_bytes, double operations_count)
    : elapsed (elapsed_arg),
      effective_bandwidth (load_store_bytes / (elapsed_arg * giga)),
      computational_throughput (operations_count / (elapsed_arg * giga)),
      matrix_format (std::move (format))
  {
  }

  measurement_class (const measurement_class &) = default;
  measurement_class &operator= (const measurement_class &o)
  {
    elapsed = o.elapsed;
    effective_bandwidth = o.effective_bandwidth;
    computational_throughput = o.computational_throughput;
    matrix_format = o.matrix_format;
    measurements_count = o.measurements_count;
    return *this;
  }

  double get_elapsed () const { return elapsed; }
  double get_effective_bandwidth () const { return effective_bandwidth; }
  double get_computational_throughput () const { return computational_throughput; }
  const std::string &get_format () const { return matrix_format; }

  measurement_class &operator+= (const measurement_class &rhs)
  {
    elapsed += rhs.get_elapsed ();
    effective_bandwidth += rhs.get_effective_bandwidth ();
    computational_throughput += rhs.get_computational_throughput ();
    matrix_format = rhs.get_format ();
    measurements_count++;
    return *this;
  }

  void finalize ()
  {
    if (measurements_count == 0)
      return;
    elapsed /= measurements_count;
    effective_bandwidth /= measurements_count;
    computational_throughput /= measurements_count;
  }

private:
  double elapsed{};
  double effective_bandwidth{};
  double computational_throughput{};
  std::string matrix_format;
  unsigned int measurements_count{};
};

template <typename data_type>
void compare_results (unsigned int y_size, const data_type *a, const data_type *b)
{
  data_type diff = 0, norm = 0;
  for (unsigned int i = 0; i < y_size; i++)
    {
      const data_type d = a[i] - b[i];
      diff += d * d;
      norm += b[i] * b[i];
    }
  const data_type error = diff / norm;
  if (error > 1e-9)
    {
      std::cerr << "ERROR: " << error << std::endl;
      for (unsigned int i = 0; i < y_size; i++)
        if (std::abs (a[i] - b[i]) > 1e-8)
          {
            std::cerr << "a[" << i << "] = " << a[i] << "; b[" << i << "] = " << b[i] << std::endl;
            break;
          }
    }
  std::cerr.flush ();
}

#endif // BMFP_MEASUREMENT_CLASS_H
