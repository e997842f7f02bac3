#pragma once
#include <functional>
namespace boost { template <typename R> using function0 = std::function<R()>; }
