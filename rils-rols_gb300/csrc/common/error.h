// Thread-local error text shared by the device runtime and the host driver.
#pragma once
#include <string>

namespace rrc {
void set_error(const std::string& msg);
const char* get_error();
}  // namespace rrc
