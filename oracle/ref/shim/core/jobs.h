#pragma once
namespace evolving_graphs {
class Jobs {};
}
