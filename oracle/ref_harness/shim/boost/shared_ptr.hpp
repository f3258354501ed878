// Test-harness shim: maps the boost smart pointer the reference uses onto std::.
// Part of the oracle harness only; never linked into the product library.
#pragma once
#include <memory>
#include <cassert>
#include <cstring>
#include <cstdlib>
#include <algorithm>
namespace boost {
using std::shared_ptr;  // same entity as std::shared_ptr, so using-directives for both namespaces stay unambiguous
}
