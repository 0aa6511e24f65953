#include "../range.hpp"
