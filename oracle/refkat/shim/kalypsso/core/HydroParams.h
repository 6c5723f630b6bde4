// Stub: the models headers include this file but use nothing from it.
#pragma once
