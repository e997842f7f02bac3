#pragma once
#include <type_traits>
