#pragma once
#include "../archive/archive_stub.hpp"
