#pragma once
#include <mutex>
namespace boost { struct mutex : std::mutex { typedef std::lock_guard<std::mutex> scoped_lock; }; }
