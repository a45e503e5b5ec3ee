/* Minimal stand-in for a TensorFlow header so the reference's CPU operator
 * sources compile without TensorFlow: they only need tensorflow::int64. */
#pragma once
namespace tensorflow { typedef long long int64; }
