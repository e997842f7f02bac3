#pragma once
#include <condition_variable>
