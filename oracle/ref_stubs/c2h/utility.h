#pragma once
#include <c2h/catch2_test_helper.h>
