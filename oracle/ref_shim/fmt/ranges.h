// Stand-in (test infrastructure for oracle/_ref).
#pragma once
#include <fmt/format.h>
