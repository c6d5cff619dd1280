/*
 * Minimal stand-in for <Python.h>, used ONLY to compile the reference's
 * unmodified generator/simulator sources into the test oracle (oracle/_ref).
 *
 * The reference raises Python UserWarnings from C++ via PyErr_WarnEx
 * (src/simulation/generator.cpp:215,357; src/simulation/simulator.cpp:294,300).
 * Here the call only bumps a thread-safe counter per message so the harness
 * can report which warnings fired; it is safe from OpenMP worker threads.
 */
#ifndef ORACLE_STUB_PYTHON_H_
#define ORACLE_STUB_PYTHON_H_

#include <atomic>
#include <cstring>

typedef long Py_ssize_t;
typedef void PyObject;

#define PyExc_UserWarning ((PyObject *)nullptr)

/* Counters live in ref_harness.cpp. */
extern std::atomic<long> g_oracle_warn_overlap;
extern std::atomic<long> g_oracle_warn_single_point;
extern std::atomic<long> g_oracle_warn_zero_axis;
extern std::atomic<long> g_oracle_warn_not_normalized;
extern std::atomic<long> g_oracle_warn_empty_light;
extern std::atomic<long> g_oracle_warn_other;

inline int PyErr_WarnEx(PyObject *, const char *msg, Py_ssize_t) {
   if (std::strstr(msg, "overlap"))
      g_oracle_warn_overlap++;
   else if (std::strstr(msg, "single point"))
      g_oracle_warn_single_point++;
   else if (std::strstr(msg, "is 0 for tissue"))
      g_oracle_warn_zero_axis++;
   else if (std::strstr(msg, "not normalized"))
      g_oracle_warn_not_normalized++;
   else if (std::strstr(msg, "light_positions is empty"))
      g_oracle_warn_empty_light++;
   else
      g_oracle_warn_other++;
   return 0;
}

#endif
