#pragma once
// Empty stand-in: the culling and transform sources include this header but use nothing from it.
