#pragma once
#include "archive_stub.hpp"
