#pragma once
#define FRIEND_TEST(test_case_name, test_name)
